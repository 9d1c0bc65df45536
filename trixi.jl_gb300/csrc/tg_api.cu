// C ABI of the GB300 DGSEM hot path (declared in include/trixi_gb300.h).
//
// A context owns, in HBM: two FP64 solution buffers (the stage kernel reads
// one and writes the other, since neighbour traces must come from the
// pre-stage state), the 2N register u_tmp (FP64, or FP32 in mixed mode),
// the face-neighbour table, the inverse Jacobians, the node coordinates
// along each axis (source terms), the indicator arrays, a device clock
// (t, dt, CFL reduction) and a status word.  A time step is one CUDA graph:
// clock_begin -> 5 fused stage kernels -> clock_end, with no host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/trixi_gb300.h"
#include "tg_clock.cuh"
#include "tg_internal.h"
#include "tg_curved.cuh"
#include "tg_mixed.cuh"

namespace tg {

// Declared per instantiation unit (tg_inst_*.cu).
#define TG_DECL(D, R, V)                                                                 \
  int launch_element_##D##d_##R##_##V(int N, int epb, const DgParams& P, const StageArgs& A, \
                                      cudaStream_t s);
TG_DECL(2, f64, weak) TG_DECL(2, f64, fd) TG_DECL(2, f64, hg)
TG_DECL(3, f64, weak) TG_DECL(3, f64, fd) TG_DECL(3, f64, hg)
#undef TG_DECL
#define TG_DECLM(D, V)                                                              \
  int launch_mixed_##D##d_##V(int N, int epb, const MixedParams& P, const MixedArgs& A, \
                              cudaStream_t s);
TG_DECLM(2, weak) TG_DECLM(2, fd) TG_DECLM(2, hg)
TG_DECLM(3, weak) TG_DECLM(3, fd) TG_DECLM(3, hg)
#undef TG_DECLM
int launch_indicator_2d_f64_hg(int N, const DgParams& P, const double* u, void* a, cudaStream_t s);
int launch_indicator_3d_f64_hg(int N, const DgParams& P, const double* u, void* a, cudaStream_t s);
int launch_indicator_mixed_2(int N, const MixedParams& P, const float2* u, float* a, cudaStream_t s);
int launch_hg_alpha_rp(int N, const MixedParams& P, const float* rp, float* alpha, cudaStream_t s);
int launch_indicator_mixed_3(int N, const MixedParams& P, const float2* u, float* a, cudaStream_t s);

int launch_element(int D, int N, bool fp64, int vi, int epb, const DgParams& P,
                   const StageArgs& A, cudaStream_t s) {
  typedef int (*Fn)(int, int, const DgParams&, const StageArgs&, cudaStream_t);
  static const Fn table[2][3] = {
      {launch_element_2d_f64_weak, launch_element_2d_f64_fd, launch_element_2d_f64_hg},
      {launch_element_3d_f64_weak, launch_element_3d_f64_fd, launch_element_3d_f64_hg}};
  if (D < 2 || D > 3 || vi < 0 || vi > 2 || !fp64) return -2;
  return table[D - 2][vi](N, epb, P, A, s);
}

static int launch_mixed(int D, int N, int vi, int epb, const MixedParams& P, const MixedArgs& A,
                        cudaStream_t s) {
  typedef int (*Fn)(int, int, const MixedParams&, const MixedArgs&, cudaStream_t);
  static const Fn table[2][3] = {{launch_mixed_2d_weak, launch_mixed_2d_fd, launch_mixed_2d_hg},
                                 {launch_mixed_3d_weak, launch_mixed_3d_fd, launch_mixed_3d_hg}};
  if (D < 2 || D > 3 || vi < 0 || vi > 2) return -2;
  return table[D - 2][vi](N, epb, P, A, s);
}

int launch_indicator(int D, int N, bool fp64, const DgParams& P, const double* u,
                     void* alpha_raw, cudaStream_t s) {
  if (!fp64) return -2;
  return D == 2 ? launch_indicator_2d_f64_hg(N, P, u, alpha_raw, s)
                : launch_indicator_3d_f64_hg(N, P, u, alpha_raw, s);
}

int default_epb(int D, int N) {
  if (D == 2) {
    switch (N) {
      case 2: return 64;
      case 3: return 28;
      case 4: return 16;
      case 5: return 10;
      case 6: return 7;
    }
  } else {
    switch (N) {
      case 2: return 32;
      case 3: return 9;
      case 4: return 4;
      case 5: return 2;
    }
  }
  return 0;
}

// Elements per block of the mixed-precision kernel (threads = EPB x lines per element).
int default_epb_mixed(int D, int N) {
  if (D == 2) {
    switch (N) {
      case 2: return 32;
      case 3: return 32;
      case 4: return 16;
      case 5: return 16;
      case 6: return 16;
    }
  } else {
    switch (N) {
      case 2: return 16;
      case 3: return 8;
      case 4: return 4;
      case 5: return 2;
    }
  }
  return 0;
}

bool supported_epb_mixed(int D, int N, int epb) {
  if (epb == default_epb_mixed(D, N)) return true;
  if (D == 2 && N == 4) return epb == 8 || epb == 32;
  if (D == 3 && N == 4) return epb == 2 || epb == 8;
  return false;
}

bool supported_epb(int D, int N, int epb) {
  if (epb == default_epb(D, N)) return true;
  if (D == 2 && N == 4) return epb == 8 || epb == 32;
  if (D == 3 && N == 4) return epb == 2 || epb == 8;
  return false;
}

// ---------------------------------------------------------------------------
// Small kernels: CFL reduction, clock, integrals, smoothing
// ---------------------------------------------------------------------------

// FP64 <-> float-float conversions of the state (the mixed path's boundary).
// The FP64 pipe of this GPU runs at 1/62 of the FP32 rate, and a conversion
// between float and double is an FP64-pipe instruction, so the conversions of
// a whole state were bound by that pipe, not by HBM.  They are done here with
// integer operations on the IEEE-754 bit patterns where the values allow it,
// with results identical to the conversion instructions, and with those
// instructions for the rest (zeros, subnormals, infinities, NaN, extreme
// exponents).

// (double)f, exact: a normal float's exponent is rebiased (127 -> 1023) and its
// 23-bit fraction shifted into the top of the 52-bit one.
__device__ __forceinline__ double widen_f32(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e - 1u < 254u)
    return __longlong_as_double((long long)(((uint64_t)(b & 0x80000000u) << 32) |
                                            ((uint64_t)(e + 896u) << 52) |
                                            ((uint64_t)(b & 0x7fffffu) << 29)));
  if ((b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((uint64_t)b << 32));
  return (double)f;  // subnormal, infinity, NaN
}

// hi = (float)x rounded to nearest even, lo = (float)(x - hi), as
// __double2float_rn(x) and __double2float_rn(x - (double)hi).  For a binary
// exponent E of x in [-74, 126], hi's fraction is x's top 23 fraction bits
// rounded to nearest even on the 29 dropped bits r (a carry into the
// exponent is the correct rounding); x - hi is exactly +-(r or r - 2^29) *
// 2^(E-52), whose rounding to float is that integer's rounding to 24 bits
// (__int2float_rn) times 2^(E-52), a normal float in this exponent range, so
// the product is exact.
__device__ __forceinline__ float2 split_f64(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;  // biased exponent, 1023 + E
  if (e - 949u <= 200u) {                           // E in [-74, 126]
    const uint32_t keep = (uint32_t)(b >> 29) & 0x7fffffu;
    const uint32_t rem = (uint32_t)b & 0x1fffffffu;
    const uint32_t up = (rem > 0x10000000u || (rem == 0x10000000u && (keep & 1u))) ? 1u : 0u;
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t hb = (sign | ((e - 896u) << 23) | keep) + up;
    int32_t r = (int32_t)rem - (int32_t)(up << 29);  // |x| - |hi| in units of 2^(E-52)
    if (sign) r = -r;                                 // x - hi (+0 when it vanishes)
    const float scale = __uint_as_float((e - 949u + 1u) << 23);  // 2^(E-52), E-52 >= -126
    return make_float2(__uint_as_float(hb), __fmul_rn(__int2float_rn(r), scale));
  }
  const float hi = __double2float_rn(x);
  return make_float2(hi, __double2float_rn(x - (double)hi));
}

__device__ __forceinline__ double state_f64(double x) { return x; }
__device__ __forceinline__ double state_f64(float2 x) { return widen_f32(x.x) + widen_f32(x.y); }

__global__ void to_ff_kernel(const double* __restrict__ in, float2* __restrict__ out, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = split_f64(in[k]);
}

// The same with two values per thread and 16-byte loads and stores (n2 = n / 2
// pairs; `in` 16-byte aligned): a warp reads and writes 512 contiguous bytes.
__global__ void to_ff2_kernel(const double2* __restrict__ in, float4* __restrict__ out, int64_t n2) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n2;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = in[k];
    const float2 a = split_f64(x.x), b = split_f64(x.y);
    out[k] = make_float4(a.x, a.y, b.x, b.y);
  }
}
// to_ff_kernel for a 2D state (4 values per node) that also writes rho*p of
// every node from the hi parts, with the stage kernels' arithmetic
__global__ void to_ff_rp_kernel(const double* __restrict__ in, float2* __restrict__ out,
                                int64_t nnodes, float gamma, float* __restrict__ rp) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnodes;
       k += (int64_t)gridDim.x * blockDim.x) {
    float hi[4], lo[4];
    for (int v = 0; v < 4; ++v) {  // 8-byte loads: `in` may be a caller's host buffer
      const float2 f = split_f64(in[4 * k + v]);
      hi[v] = f.x;
      lo[v] = f.y;
    }
    reinterpret_cast<float4*>(out)[2 * k] = make_float4(hi[0], lo[0], hi[1], lo[1]);
    reinterpret_cast<float4*>(out)[2 * k + 1] = make_float4(hi[2], lo[2], hi[3], lo[3]);
    rp[k] = Euler<2, float>::density_pressure(hi, gamma);
  }
}

template <int D>
__device__ __forceinline__ bool node_speeds_ff(const float* hi, float gamma, float* ml);
__device__ __forceinline__ void block_speed_max(unsigned long long mine,
                                                unsigned long long* __restrict__ speed_bits);

// to_ff_rp_kernel fused with the CFL reduction of the imported state (the
// reduction max_speed_ff_kernel<2> makes, same arithmetic, same result): a
// 2D element's NN nodes (NN a power of two <= 16) are NN consecutive threads,
// which combine their speeds by shuffles within their lane group; the block
// maximum goes to speed_bits by one atomicMax.  speed_bits must hold its
// initial value (speed_reset_kernel) before the launch.
template <int NN>
__global__ void __launch_bounds__(256) to_ff_rp_speed_kernel(
    const double* __restrict__ in, float2* __restrict__ out, int64_t nnodes, float gamma_rp,
    float* __restrict__ rp, float gamma, const float* __restrict__ inv_jac,
    unsigned long long* __restrict__ speed_bits, int32_t* __restrict__ status) {
  static_assert(NN >= 1 && NN <= 16 && (NN & (NN - 1)) == 0, "lane groups of NN threads");
  const int lane = threadIdx.x & 31;
  const unsigned gmask = ((1u << NN) - 1u) << (lane & ~(NN - 1));
  unsigned long long best = 0;
  bool bad = false;
  // the grid stride is a multiple of NN, so an element's threads stay together
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnodes;
       k += (int64_t)gridDim.x * blockDim.x) {
    float hi[4], lo[4];
    for (int v = 0; v < 4; ++v) {  // 8-byte loads: `in` may be a caller's host buffer
      const float2 f = split_f64(in[4 * k + v]);
      hi[v] = f.x;
      lo[v] = f.y;
    }
    reinterpret_cast<float4*>(out)[2 * k] = make_float4(hi[0], lo[0], hi[1], lo[1]);
    reinterpret_cast<float4*>(out)[2 * k + 1] = make_float4(hi[2], lo[2], hi[3], lo[3]);
    rp[k] = Euler<2, float>::density_pressure(hi, gamma_rp);
    float ml[2];
    bad |= node_speeds_ff<2>(hi, gamma, ml);
    for (int d = 0; d < 2; ++d)
      for (int o = NN / 2; o > 0; o >>= 1) ml[d] = fmaxf(ml[d], __shfl_xor_sync(gmask, ml[d], o));
    if ((lane & (NN - 1)) == 0) {
      float sum = 0;
      for (int d = 0; d < 2; ++d) sum += ml[d];
      const float sp = inv_jac[k / NN] * sum;
      if (sp == sp) {
        const unsigned long long b = (unsigned long long)__double_as_longlong((double)sp);
        best = b > best ? b : best;
      } else {
        bad = true;
      }
    }
  }
  if (bad) atomicOr(status, 2);
  block_speed_max(best, speed_bits);
}

// to_ff_rp_speed_kernel<16> with 16-byte loads and stores (`in` 16-byte
// aligned): a thread converts two values of a node (lane pair: values 0-1 and
// 2-3), the pair exchanges its hi parts by shuffles, and a warp covers one
// element (16 nodes) per pass, so the element's speed reduction is a warp
// reduction.  Same arithmetic, same results.
__global__ void __launch_bounds__(256) to_ff_rp_speed_pair_kernel(
    const double2* __restrict__ in, float4* __restrict__ out, int64_t nnodes, float gamma_rp,
    float* __restrict__ rp, float gamma, const float* __restrict__ inv_jac,
    unsigned long long* __restrict__ speed_bits, int32_t* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int64_t npairs = 2 * nnodes;  // a multiple of 32: elements of 16 nodes
  unsigned long long best = 0;
  bool bad = false;
  // blockDim and the grid stride are multiples of 32: a warp's 32 pairs are
  // one element, and the loop condition is warp-uniform
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npairs;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = in[p];
    const float2 a = split_f64(x.x), b = split_f64(x.y);
    out[p] = make_float4(a.x, a.y, b.x, b.y);
    const float oa = __shfl_xor_sync(0xffffffffu, a.x, 1);
    const float ob = __shfl_xor_sync(0xffffffffu, b.x, 1);
    const bool first = (lane & 1) == 0;
    float hi[4];
    hi[0] = first ? a.x : oa;
    hi[1] = first ? b.x : ob;
    hi[2] = first ? oa : a.x;
    hi[3] = first ? ob : b.x;
    float ml[2] = {0.0f, 0.0f};
    if (first) {
      rp[p >> 1] = Euler<2, float>::density_pressure(hi, gamma_rp);
      bad |= node_speeds_ff<2>(hi, gamma, ml);
    }
    for (int d = 0; d < 2; ++d)
      for (int o = 16; o > 0; o >>= 1) ml[d] = fmaxf(ml[d], __shfl_xor_sync(0xffffffffu, ml[d], o));
    if (lane == 0) {
      float sum = 0;
      for (int d = 0; d < 2; ++d) sum += ml[d];
      const float sp = inv_jac[p >> 5] * sum;
      if (sp == sp) {
        const unsigned long long bits = (unsigned long long)__double_as_longlong((double)sp);
        best = bits > best ? bits : best;
      } else {
        bad = true;
      }
    }
  }
  if (bad) atomicOr(status, 2);
  block_speed_max(best, speed_bits);
}

// rho*p of every node from the hi parts of a float-float state (nv values per
// node), with the stage kernels' arithmetic
__global__ void rho_p_ff_kernel(const float2* __restrict__ u, int64_t nnodes, int nv, float gamma,
                                float* __restrict__ rp) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnodes;
       k += (int64_t)gridDim.x * blockDim.x) {
    float hi[5];
    for (int v = 0; v < nv; ++v) hi[v] = u[k * nv + v].x;
    rp[k] = nv == 4 ? Euler<2, float>::density_pressure(hi, gamma)
                    : Euler<3, float>::density_pressure(hi, gamma);
  }
}

__global__ void from_ff_kernel(const float2* __restrict__ in, double* __restrict__ out, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = state_f64(in[k]);
}

// The same with two values per thread and 16-byte loads and stores (`out`
// 16-byte aligned).
__global__ void from_ff2_kernel(const float4* __restrict__ in, double2* __restrict__ out, int64_t n2) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n2;
       k += (int64_t)gridDim.x * blockDim.x) {
    const float4 x = in[k];
    out[k] = make_double2(state_f64(make_float2(x.x, x.y)), state_f64(make_float2(x.z, x.w)));
  }
}

// max_dt's reduction (stepsize_dg2d.jl:8-30): max_e invJ_e * sum_d max_nodes lambda_d.
// max_dt reductions (stepsize_dg{2,3}d.jl): one warp per element, lanes over
// its nodes (consecutive lanes read consecutive nodes), a warp max per
// direction, then lane 0 adds the directions and updates the global maximum.
// Block maximum of the lanes' speed bits (positive doubles order like their
// bit patterns) into one atomicMax per block: the warps walk the elements with
// a grid stride, so the whole reduction is one atomic per block instead of one
// per element on a single address.
__device__ __forceinline__ void block_speed_max(unsigned long long mine,
                                                unsigned long long* __restrict__ speed_bits) {
  __shared__ unsigned long long s_max[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, mine, o);
    mine = other > mine ? other : mine;
  }
  if (lane == 0) s_max[warp] = mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long m = s_max[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = s_max[w] > m ? s_max[w] : m;
    if (m) atomicMax(speed_bits, m);
  }
}

// max_dt's reduction (stepsize_dg2d.jl:8-30, stepsize_dg3d.jl): per element the
// sum over directions of the node maxima of |v_d| + c, times the inverse
// Jacobian; one warp per element at a time, 4 warps per block.
template <int D, typename TS>
__global__ void __launch_bounds__(128) max_speed_kernel(const TS* __restrict__ u,
                                                        const double* __restrict__ inv_jac,
                                                        int64_t E, int NN, double gamma,
                                                        unsigned long long* __restrict__ speed_bits,
                                                        int32_t* __restrict__ status) {
  constexpr int NV = D + 2;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  unsigned long long best = 0;
  bool bad = false;
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < E;
       e += nwarps) {
    double ml[D];
    for (int d = 0; d < D; ++d) ml[d] = 0;
    for (int q = lane; q < NN; q += 32) {
      const TS* p = u + ((size_t)e * NN + q) * NV;
      double uu[NV], w[NV];
      for (int v = 0; v < NV; ++v) uu[v] = state_f64(p[v]);
      Euler<D, double>::cons2prim(uu, w, gamma);
      const double c = sqrt(gamma * w[NV - 1] / w[0]);
      bad |= !(w[0] > 0) || !(w[NV - 1] > 0);
      for (int d = 0; d < D; ++d) ml[d] = fmax(ml[d], fabs(w[1 + d]) + c);
    }
    for (int d = 0; d < D; ++d)
      for (int o = 16; o > 0; o >>= 1) ml[d] = fmax(ml[d], __shfl_xor_sync(0xffffffffu, ml[d], o));
    double sum = ml[0];
    for (int d = 1; d < D; ++d) sum += ml[d];
    const double sp = inv_jac[e] * sum;
    if (sp == sp) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(sp);
      best = b > best ? b : best;
    } else if (lane == 0) {
      bad = true;
    }
  }
  if (bad) atomicOr(status, 2);
  block_speed_max(best, speed_bits);
}

// Per-node wave speeds |v_d| + c of a mixed context's CFL reduction from the
// hi parts of the state (FP32 primitives and sound speed); a NaN speed (a
// non-positive density or pressure) counts as 0 and is flagged.
template <int D>
__device__ __forceinline__ bool node_speeds_ff(const float* hi, float gamma, float* ml) {
  constexpr int NV = D + 2;
  float w[NV];
  Euler<D, float>::cons2prim(hi, w, gamma);
  const float cs = sqrtf(gamma * w[NV - 1] / w[0]);
  for (int d = 0; d < D; ++d) {
    const float lam = fabsf(w[1 + d]) + cs;
    ml[d] = lam == lam ? lam : 0.0f;
  }
  return !(w[0] > 0.0f) || !(w[NV - 1] > 0.0f);
}

// The same reduction for a mixed context in the FP32 arithmetic its stage
// kernel uses for the wave speed of the updated state (hi parts, FP32
// primitives and sound speed, FP32 inverse Jacobian), so that the first dt
// after an upload is computed like every later one.
template <int D>
__global__ void __launch_bounds__(128) max_speed_ff_kernel(const float2* __restrict__ u,
                                                           const float* __restrict__ inv_jac,
                                                           int64_t E, int NN, float gamma,
                                                           unsigned long long* __restrict__ speed_bits,
                                                           int32_t* __restrict__ status) {
  constexpr int NV = D + 2;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  unsigned long long best = 0;
  bool bad = false;
  for (int64_t e = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < E;
       e += nwarps) {
    float ml[D];
    for (int d = 0; d < D; ++d) ml[d] = 0.0f;
    for (int q = lane; q < NN; q += 32) {
      const float2* p = u + ((size_t)e * NN + q) * NV;
      float hi[NV], lam[D];
      for (int v = 0; v < NV; ++v) hi[v] = p[v].x;
      bad |= node_speeds_ff<D>(hi, gamma, lam);
      for (int d = 0; d < D; ++d) ml[d] = fmaxf(ml[d], lam[d]);
    }
    for (int d = 0; d < D; ++d)
      for (int o = 16; o > 0; o >>= 1) ml[d] = fmaxf(ml[d], __shfl_xor_sync(0xffffffffu, ml[d], o));
    float sum = 0;
    for (int d = 0; d < D; ++d) sum += ml[d];
    const float sp = inv_jac[e] * sum;
    if (sp == sp) {
      const unsigned long long b = (unsigned long long)__double_as_longlong((double)sp);
      best = b > best ? b : best;
    } else if (lane == 0) {
      bad = true;
    }
  }
  if (bad) atomicOr(status, 2);
  block_speed_max(best, speed_bits);
}

__global__ void speed_reset_kernel(unsigned long long* speed_bits) {
  // nextfloat(0.0): max_dt starts its reduction there (stepsize_dg2d.jl:12)
  *speed_bits = 1ull;
}

// initialize! of StepsizeCallback: dt = cfl * max_dt(u)
__global__ void clock_init_kernel(Clock* c, double t, double t_end, double cfl, int n) {
  c->t = t;
  c->t_end = t_end;
  c->cfl = cfl;
  const double speed = __longlong_as_double((long long)c->speed_bits);
  c->dt = cfl * (2.0 / (n * speed));
  c->skip = 0;
  c->finalstep = 0;
  c->finished = 0;
  c->nan_dt = 0;
  c->steps = 0;
}

__global__ void clock_set_kernel(Clock* c, double t, double dt) {
  c->t = t;
  c->dt = dt;
  c->t_end = INFINITY;
  c->skip = 0;
  c->finalstep = 0;
  c->finished = 0;
  stage_phases(c);
}

__global__ void clock_config_kernel(Clock* c, double t_end, double cfl) {
  c->t_end = t_end;
  c->cfl = cfl;
  c->finished = 0;
  c->finalstep = 0;
}

__global__ void clock_begin_kernel(Clock* c) { clock_begin_warp(c); }

__global__ void clock_end_kernel(Clock* c, int n) { clock_end(c, n); }

// Per-element FP64 integrals (integrate_via_indices, analysis_dg2d.jl:313-336):
// conserved totals, mathematical entropy (compressible_euler_2d.jl:2236-2255)
// and kinetic energy (:2297-2300).
template <int D, typename TS>
__global__ void element_integrals_kernel(const TS* __restrict__ u,
                                         const double* __restrict__ inv_jac,
                                         const double* __restrict__ weights, int64_t E, int N,
                                         double gamma, double* __restrict__ partial) {
  constexpr int NV = D + 2;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  int NN = N * N;
  if (D == 3) NN *= N;
  double vj = 1.0 / inv_jac[e];
  vj = D == 2 ? vj * vj : vj * vj * vj;
  double acc[NV + 2];
  for (int k = 0; k < NV + 2; ++k) acc[k] = 0;
  for (int q = 0; q < NN; ++q) {
    const int i = q % N, j = (q / N) % N, k = q / (N * N);
    double w = weights[i] * weights[j];
    if (D == 3) w *= weights[k];
    double p[NV];
    for (int v = 0; v < NV; ++v) p[v] = state_f64(u[((size_t)e * NN + q) * NV + v]);
    double m2 = 0;
    for (int d = 0; d < D; ++d) m2 += p[1 + d] * p[1 + d];
    for (int v = 0; v < NV; ++v) acc[v] += vj * w * p[v];
    const double pr = (gamma - 1) * (p[NV - 1] - 0.5 * m2 / p[0]);
    const double s = log(pr) - gamma * log(p[0]);
    acc[NV] += vj * w * (-s * p[0] / (gamma - 1));
    acc[NV + 1] += vj * w * (m2 / (2 * p[0]));
  }
  for (int k = 0; k < NV + 2; ++k) partial[(size_t)e * (NV + 2) + k] = acc[k];
}

// Per-element FP64 entropy production sum_nodes w J cons2entropy(u) . du
// (analysis_dg2d.jl:460-472; cons2entropy, compressible_euler_2d.jl:2049-2066).
template <int D>
__global__ void element_entropy_kernel(const double* __restrict__ u, const double* __restrict__ du,
                                       const double* __restrict__ inv_jac,
                                       const double* __restrict__ weights, int64_t E, int N,
                                       double gamma, double* __restrict__ partial) {
  constexpr int NV = D + 2;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  int NN = N * N;
  if (D == 3) NN *= N;
  double vj = 1.0 / inv_jac[e];
  vj = D == 2 ? vj * vj : vj * vj * vj;
  double acc = 0, vol = 0;
  for (int q = 0; q < NN; ++q) {
    const int i = q % N, j = (q / N) % N, k = q / (N * N);
    double w = weights[i] * weights[j];
    if (D == 3) w *= weights[k];
    const double* p = u + ((size_t)e * NN + q) * NV;
    const double* dp = du + ((size_t)e * NN + q) * NV;
    double v[D], v2 = 0;
    for (int d = 0; d < D; ++d) {
      v[d] = p[1 + d] / p[0];
      v2 += v[d] * v[d];
    }
    const double pr = (gamma - 1) * (p[NV - 1] - 0.5 * p[0] * v2);
    const double s = log(pr) - gamma * log(p[0]);
    const double rho_p = p[0] / pr;
    double dot = ((gamma - s) / (gamma - 1) - 0.5 * rho_p * v2) * dp[0];
    for (int d = 0; d < D; ++d) dot += rho_p * v[d] * dp[1 + d];
    dot += -rho_p * dp[NV - 1];
    acc += vj * w * dot;
    vol += vj * w;
  }
  partial[2 * e] = acc;
  partial[2 * e + 1] = vol;
}

// Deterministic sum of partial[E][K] over elements (one block).
__global__ void sum_rows_kernel(const double* __restrict__ partial, int64_t E, int K,
                                double* __restrict__ out) {
  extern __shared__ double sh[];
  for (int k = 0; k < K; ++k) {
    double s = 0;
    for (int64_t e = threadIdx.x; e < E; e += blockDim.x) s += partial[(size_t)e * K + k];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = sh[0];
    __syncthreads();
  }
}

// calc_error_norms (analysis_dg2d.jl:95-139, analysis_dg3d.jl:123-...): per
// element, the state and the node coordinates interpolated to the analyzer's
// NA^D nodes dimension by dimension (multiply_dimensionwise!, x then y then z,
// each sum in node order as the reference), the exact solution (a device
// initial condition) there, and per variable the Jacobian-weighted sum of
// squared differences and their maximum.  One block per element; the two
// ping-pong buffers hold NC = NV + D values per node.
struct ErrorNormArgs {
  int N, NA, ic;
  double par[4];
  double t, gamma;
  double avand[MAXN * (2 * MAXN - 1)];  // [NA][N], row-major
  double aw[2 * MAXN - 1];
};

template <int D, typename TS>
__global__ void __launch_bounds__(128) error_norms_kernel(const TS* __restrict__ u,
                                                          const double* __restrict__ xline,
                                                          const double* __restrict__ inv_jac,
                                                          const ErrorNormArgs A,
                                                          double* __restrict__ partial) {
  constexpr int NV = D + 2, NC = NV + D;
  extern __shared__ double esm[];
  const int N = A.N, NA = A.NA;
  int nn = N, nna = NA;
  for (int d = 1; d < D; ++d) nn *= N, nna *= NA;
  double* cur = esm;
  double* nxt = esm + (size_t)nna * NC;
  double* red = nxt + (size_t)nna * NC;  // [blockDim][2 NV]
  const int64_t e = blockIdx.x;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    for (int v = 0; v < NV; ++v) cur[q * NC + v] = state_f64(u[((size_t)e * nn + q) * NV + v]);
    const int idx[3] = {q % N, (q / N) % N, q / (N * N)};
    for (int d = 0; d < D; ++d) cur[q * NC + NV + d] = xline[((size_t)e * D + d) * N + idx[d]];
  }
  __syncthreads();
  int dims[3] = {N, N, N};
  for (int d = 0; d < D; ++d) {
    int so[3] = {dims[0], dims[1], dims[2]};
    so[d] = NA;
    int tot = 1;
    for (int q = 0; q < D; ++q) tot *= so[q];
    for (int o = threadIdx.x; o < tot; o += blockDim.x) {
      const int ii[3] = {o % so[0], (o / so[0]) % so[1], o / (so[0] * so[1])};
      for (int v = 0; v < NC; ++v) {
        double r = 0;
        for (int k = 0; k < N; ++k) {
          int src[3] = {ii[0], ii[1], ii[2]};
          src[d] = k;
          const int si = src[0] + dims[0] * (src[1] + dims[1] * src[2]);
          r += A.avand[ii[d] * N + k] * cur[si * NC + v];
        }
        nxt[o * NC + v] = r;
      }
    }
    __syncthreads();
    double* t = cur;
    cur = nxt;
    nxt = t;
    dims[d] = NA;
  }
  double vj = 1.0 / inv_jac[e];
  vj = D == 2 ? vj * vj : vj * vj * vj;
  double loc[NV], mx[NV];
  for (int v = 0; v < NV; ++v) loc[v] = mx[v] = 0.0;
  for (int o = threadIdx.x; o < nna; o += blockDim.x) {
    const int idx[3] = {o % NA, (o / NA) % NA, o / (NA * NA)};
    double w = A.aw[idx[0]] * A.aw[idx[1]];
    if (D == 3) w *= A.aw[idx[2]];
    double ue[NV];
    boundary_value<D>(A.ic, A.par, &cur[o * NC + NV], A.t, A.gamma, ue);
    for (int v = 0; v < NV; ++v) {
      const double diff = ue[v] - cur[o * NC + v];
      loc[v] += diff * diff * (w * vj);
      mx[v] = fmax(mx[v], fabs(diff));
    }
  }
  for (int v = 0; v < NV; ++v) {
    red[threadIdx.x * 2 * NV + v] = loc[v];
    red[threadIdx.x * 2 * NV + NV + v] = mx[v];
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // in thread order: deterministic
    for (int v = 0; v < NV; ++v) {
      double sum = 0, m = 0;
      for (int k = 0; k < (int)blockDim.x; ++k) {
        sum += red[k * 2 * NV + v];
        m = fmax(m, red[k * 2 * NV + NV + v]);
      }
      partial[(size_t)e * 2 * NV + v] = sum;
      partial[(size_t)e * 2 * NV + NV + v] = m;
    }
  }
}

// Column sums (k < K) and maxima (K <= k < 2K) of partial[E][2K], each
// thread's share in element order and then a fixed tree: deterministic.
__global__ void sum_max_rows_kernel(const double* __restrict__ partial, int64_t E, int K,
                                    double* __restrict__ out) {
  extern __shared__ double sh[];
  for (int k = 0; k < 2 * K; ++k) {
    const bool is_max = k >= K;
    double s = 0;
    for (int64_t e = threadIdx.x; e < E; e += blockDim.x) {
      const double x = partial[(size_t)e * 2 * K + k];
      s = is_max ? fmax(s, x) : s + x;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w)
        sh[threadIdx.x] = is_max ? fmax(sh[threadIdx.x], sh[threadIdx.x + w])
                                 : sh[threadIdx.x] + sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = sh[0];
    __syncthreads();
  }
}

// Boundary pre-pass of a mixed context (calc_boundary_flux!, dg_2d.jl:795-860,
// evaluated for the stage's input state): for every node of every boundary
// face, in FP64, the Dirichlet state (the initial condition at the node and
// the stage time t + c dt) or the slip-wall flux, stored as float-float pairs
// for the stage kernel, which reads them like a neighbour's trace.
template <int D>
__global__ void boundary_ghost_kernel(const DgParams P, const float2* __restrict__ u,
                                      const int32_t* __restrict__ bface, int64_t B, int N,
                                      const Clock* clock, double c_s, double t_rhs, int mode,
                                      float2* __restrict__ ghost) {
  constexpr int NV = D + 2;
  const int NF = D == 2 ? N : N * N;
  const int NN = NF * N;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= B * NF) return;
  const int64_t b = k / NF;
  const int fn = (int)(k - b * NF);
  const int64_t e = bface[2 * b];
  const int dir = bface[2 * b + 1];
  const int d = dir >> 1, side = dir & 1;
  const int S = d == 0 ? 1 : (d == 1 ? N : N * N);
  const int node = (fn % S) + (fn / S) * S * N + (side ? (N - 1) * S : 0);
  double out[NV];
  if (P.bc[dir] == BC_SLIP_WALL) {
    const float2* p = u + ((size_t)e * NN + node) * NV;
    double ui[NV], w[NV];
    for (int v = 0; v < NV; ++v) ui[v] = (double)p[v].x + (double)p[v].y;
    Euler<D, double>::cons2prim(ui, w, P.gamma);
    const double vn = side ? w[1 + d] : -w[1 + d];  // outward normal velocity
    const double ps = slip_wall_pressure<double>(w[0], vn, w[NV - 1], P.gamma, P.inv_gamma_minus_one);
    for (int v = 0; v < NV; ++v) out[v] = 0.0;
    out[1 + d] = ps;
  } else {
    double x[D];
    for (int q = 0; q < D; ++q) {
      const int Sq = q == 0 ? 1 : (q == 1 ? N : N * N);
      x[q] = P.xline[((size_t)e * D + q) * N + (node / Sq) % N];
    }
    const double t = mode == MODE_RHS ? t_rhs : clock->t + c_s * clock->dt;
    boundary_value<D>(P.bc_ic, P.bc_par, x, t, P.gamma, out);
  }
  for (int v = 0; v < NV; ++v) {
    const float hi = (float)out[v];
    ghost[k * NV + v] = make_float2(hi, (float)(out[v] - (double)hi));
  }
}

// Mortar pre-pass (prolong2mortars! + calc_mortar_flux! +
// mortar_fluxes_to_elements!, dg_2d.jl:899-1243, dg_3d.jl:770-1335) for the
// stage's input state, in FP64, one block per mortar: the large element's
// trace is interpolated to each half (2D) or quarter (3D) face with
// forward_{lower,upper} (one matrix per face axis), the surface flux is taken
// there against the small element's trace, and the small faces' fluxes are
// projected back onto the large face with reverse_{lower,upper}.  mtab per
// mortar: the 2^(D-1) small elements (first face axis fastest), the large
// one, large side (0: large element on the negative side), orientation.
// The flux of mortar face slot m (2^(D-1) + 1) + q (q: small element q, then
// the large one) goes to out64 (FP64 contexts) or, as float-float, to
// outff at slot + ff_offset (mixed contexts, after the boundary faces).
template <int D, typename S>
__global__ void __launch_bounds__(128)
    mortar_flux_kernel(const DgParams P, const S* __restrict__ u, const int32_t* __restrict__ mtab,
                       const double* __restrict__ mmat, int64_t M, int N, int64_t ff_offset,
                       double* __restrict__ out64, float2* __restrict__ outff) {
  constexpr int NV = D + 2, NS = 1 << (D - 1);
  constexpr int MAXF = D == 2 ? MAXN : MAXN * MAXN;
  __shared__ double s_mat[4 * MAXN * MAXN];  // forward lower, upper; reverse lower, upper
  __shared__ double s_ul[MAXF * NV];         // large element's trace
  __shared__ double s_f[NS * MAXF * NV];     // fluxes on the small faces
  const int64_t m = blockIdx.x;
  if (m >= M) return;
  const int tid = threadIdx.x;
  const int NF = D == 2 ? N : N * N, NN = NF * N, NM = N * N;
  for (int k = tid; k < 4 * NM; k += blockDim.x) s_mat[k] = mmat[k];
  const int32_t* t = mtab + m * (NS + 3);
  const int ls = t[NS + 1], o = t[NS + 2];
  const int dir_large = ls == 0 ? 2 * o + 1 : 2 * o;  // large face towards the small ones
  const int dir_small = dir_large ^ 1;
  const int Sd = o == 0 ? 1 : (o == 1 ? N : N * N);
  auto face_node = [&](int fn, int dir) {
    return (fn % Sd) + (fn / Sd) * Sd * N + ((dir & 1) ? (N - 1) * Sd : 0);
  };
  auto load = [&](int64_t e, int node, double* x) {
    const S* p = u + ((size_t)e * NN + node) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      if constexpr (std::is_same<S, double>::value)
        x[v] = p[v];
      else
        x[v] = (double)p[v].x + (double)p[v].y;  // float-float pair
    }
  };
  auto store = [&](int64_t slot, int fn, const double* f) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const size_t k = ((size_t)slot * NF + fn) * NV + v;
      if (out64) {
        out64[k] = f[v];
      } else {
        const float hi = (float)f[v];
        outff[(size_t)ff_offset * NF * NV + k] = make_float2(hi, (float)(f[v] - (double)hi));
      }
    }
  };
  for (int fn = tid; fn < NF; fn += blockDim.x) {
    double x[NV];
    load(t[NS], face_node(fn, dir_large), x);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_ul[fn * NV + v] = x[v];
  }
  __syncthreads();
  const double gamma = P.gamma, igm1 = P.inv_gamma_minus_one;
  using Eu = Euler<D, double>;
  for (int it = tid; it < NS * NF; it += blockDim.x) {
    const int q = it / NF, fn = it - q * NF;
    const int i = fn % N, j = fn / N;
    const double* F1 = s_mat + (q & 1) * NM;
    const double* F2 = s_mat + ((q >> 1) & 1) * NM;
    double up[NV], us[NV], wp[NV], ws[NV], F[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) up[v] = 0.0;
    if (D == 2) {
      for (int a = 0; a < N; ++a) {
        const double c = F1[i * N + a];
#pragma unroll
        for (int v = 0; v < NV; ++v) up[v] += c * s_ul[a * NV + v];
      }
    } else {
      for (int b = 0; b < N; ++b)
        for (int a = 0; a < N; ++a) {
          const double c = F1[i * N + a] * F2[j * N + b];
#pragma unroll
          for (int v = 0; v < NV; ++v) up[v] += c * s_ul[(a + b * N) * NV + v];
        }
    }
    load(t[q], face_node(fn, dir_small), us);
    Eu::cons2prim(up, wp, gamma);
    Eu::cons2prim(us, ws, gamma);
    if (ls == 0)
      Eu::two_point(P.surface_flux, up, wp, us, ws, o, gamma, igm1, F);
    else
      Eu::two_point(P.surface_flux, us, ws, up, wp, o, gamma, igm1, F);
#pragma unroll
    for (int v = 0; v < NV; ++v) s_f[it * NV + v] = F[v];
    store(m * (NS + 1) + q, fn, F);
  }
  __syncthreads();
  for (int fn = tid; fn < NF; fn += blockDim.x) {
    const int i = fn % N, j = fn / N;
    double r[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) r[v] = 0.0;
    for (int q = 0; q < NS; ++q) {
      const double* R1 = s_mat + (2 + (q & 1)) * NM;
      const double* R2 = s_mat + (2 + ((q >> 1) & 1)) * NM;
      const double* f = s_f + (size_t)q * NF * NV;
      if (D == 2) {
        for (int a = 0; a < N; ++a) {
          const double c = R1[i * N + a];
#pragma unroll
          for (int v = 0; v < NV; ++v) r[v] += c * f[a * NV + v];
        }
      } else {
        for (int b = 0; b < N; ++b)
          for (int a = 0; a < N; ++a) {
            const double c = R1[i * N + a] * R2[j * N + b];
#pragma unroll
            for (int v = 0; v < NV; ++v) r[v] += c * f[(a + b * N) * NV + v];
          }
      }
    }
    store(m * (NS + 1) + NS, fn, r);
  }
}

// Mortar pre-pass of a mixed context: the fluxes of mortar_flux_kernel in the
// mixed kernel's deviation form.  The large element's first face node is the
// reference (Dev::make_ref on its hi part); every other state is a deviation
// from it: the large trace's in FP32, forward_{lower,upper} acting on those
// deviations (exact to their FP32 rounding, every row sums to one), and the
// small traces through Dev::make_node.  The surface flux is the element
// kernel's (Dev::two_point, F - f(w_ref)); f(w_ref) is added back in FP64 and
// reverse_{lower,upper} project the deviations F - f(w_ref) (the reverse
// rows of all small faces together sum to one).  mat32: the four matrices in
// FP32, row-major.
template <int D>
__global__ void __launch_bounds__(128)
    mortar_flux_ff_kernel(const MixedParams P, const float2* __restrict__ u,
                          const int32_t* __restrict__ mtab, const float* __restrict__ mat32,
                          int64_t M, int N, int64_t ff_offset, float2* __restrict__ outff) {
  constexpr int NV = D + 2, NS = 1 << (D - 1), PP = D + 1;
  constexpr int MAXF = D == 2 ? MAXN : MAXN * MAXN;
  using Dv = Dev<D>;
  __shared__ float s_mat[4 * MAXN * MAXN];
  __shared__ float s_dl[MAXF * NV];        // large trace - reference (FP32)
  __shared__ float s_df[NS * MAXF * NV];   // F - f(w_ref) on the small faces
  __shared__ RefState<D> s_R;
  __shared__ float s_lo[NV];               // low part of the reference node
  __shared__ double s_fref[NV];            // f(w_ref) along the mortar's orientation
  const int64_t m = blockIdx.x;
  if (m >= M) return;
  const int tid = threadIdx.x;
  const int NF = D == 2 ? N : N * N, NN = NF * N, NM = N * N;
  const EosF& eos = P.eos;
  for (int k = tid; k < 4 * NM; k += blockDim.x) s_mat[k] = mat32[k];
  const int32_t* t = mtab + m * (NS + 3);
  const int ls = t[NS + 1], o = t[NS + 2];
  const int dir_large = ls == 0 ? 2 * o + 1 : 2 * o;
  const int dir_small = dir_large ^ 1;
  const int Sd = o == 0 ? 1 : (o == 1 ? N : N * N);
  auto face_node = [&](int fn, int dir) {
    return (fn % Sd) + (fn / Sd) * Sd * N + ((dir & 1) ? (N - 1) * Sd : 0);
  };
  const float2* ul = u + (size_t)t[NS] * NN * NV;
  const float2* ur0 = ul + (size_t)face_node(0, dir_large) * NV;  // reference node
  if (tid == 0) {
    float hi[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      hi[v] = ur0[v].x;
      s_lo[v] = ur0[v].y;
    }
    RefState<D> R;
    Dv::make_ref(hi, eos, R);
    s_R = R;
    // the physical flux of the reference primitives, with the EOS constants
    // of the deviation functions
    const double rho = R.rho, p = R.p, vo = R.v[o];
    double v2 = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) v2 += (double)R.v[d] * (double)R.v[d];
    s_fref[0] = rho * vo;
#pragma unroll
    for (int d = 0; d < D; ++d) s_fref[1 + d] = rho * vo * (double)R.v[d] + (d == o ? p : 0.0);
    s_fref[PP] = (p * (double)eos.igm1 + 0.5 * rho * v2 + p) * vo;
  }
  for (int fn = tid; fn < NF; fn += blockDim.x) {
    const float2* q = ul + (size_t)face_node(fn, dir_large) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) s_dl[fn * NV + v] = (q[v].x - ur0[v].x) + (q[v].y - ur0[v].y);
  }
  __syncthreads();
  const RefState<D>& R = s_R;
  const float vro = Dv::pick(R.v, o);
  for (int it = tid; it < NS * NF; it += blockDim.x) {
    const int q = it / NF, fn = it - q * NF;
    const int i = fn % N, j = fn / N;
    const float* F1 = s_mat + (q & 1) * NM;
    const float* F2 = s_mat + ((q >> 1) & 1) * NM;
    float hp[NV], lp[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      hp[v] = R.hi[v];
      lp[v] = s_lo[v];
    }
    if (D == 2) {
      for (int a = 0; a < N; ++a) {
        const float c = F1[i * N + a];
#pragma unroll
        for (int v = 0; v < NV; ++v) lp[v] = fmaf(c, s_dl[a * NV + v], lp[v]);
      }
    } else {
      for (int b = 0; b < N; ++b)
        for (int a = 0; a < N; ++a) {
          const float c = F1[i * N + a] * F2[j * N + b];
#pragma unroll
          for (int v = 0; v < NV; ++v) lp[v] = fmaf(c, s_dl[(a + b * N) * NV + v], lp[v]);
        }
    }
    const float2* ps = u + ((size_t)t[q] * NN + face_node(fn, dir_small)) * NV;
    float hs[NV], lo_s[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      hs[v] = ps[v].x;
      lo_s[v] = ps[v].y;
    }
    Node<D> np, ns;
    Dv::make_node(hp, lp, R, eos, np);
    Dv::make_node(hs, lo_s, R, eos, ns);
    Dv::orient(np, o);
    Dv::orient(ns, o);
    float F[NV];
    if (ls == 0)
      Dv::two_point(P.surface_flux, R, np, ns, o, vro, eos, F);
    else
      Dv::two_point(P.surface_flux, R, ns, np, o, vro, eos, F);
    const size_t slot = (size_t)(ff_offset + m * (NS + 1) + q);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      s_df[it * NV + v] = F[v];
      const double x = s_fref[v] + (double)F[v];
      const float hi = (float)x;
      outff[(slot * NF + fn) * NV + v] = make_float2(hi, (float)(x - (double)hi));
    }
  }
  __syncthreads();
  for (int fn = tid; fn < NF; fn += blockDim.x) {
    const int i = fn % N, j = fn / N;
    float r[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) r[v] = 0.f;
    for (int q = 0; q < NS; ++q) {
      const float* R1 = s_mat + (2 + (q & 1)) * NM;
      const float* R2 = s_mat + (2 + ((q >> 1) & 1)) * NM;
      const float* f = s_df + (size_t)q * NF * NV;
      if (D == 2) {
        for (int a = 0; a < N; ++a) {
          const float c = R1[i * N + a];
#pragma unroll
          for (int v = 0; v < NV; ++v) r[v] = fmaf(c, f[a * NV + v], r[v]);
        }
      } else {
        for (int b = 0; b < N; ++b)
          for (int a = 0; a < N; ++a) {
            const float c = R1[i * N + a] * R2[j * N + b];
#pragma unroll
            for (int v = 0; v < NV; ++v) r[v] = fmaf(c, f[(a + b * N) * NV + v], r[v]);
          }
      }
    }
    const size_t slot = (size_t)(ff_offset + m * (NS + 1) + NS);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double x = s_fref[v] + (double)r[v];
      const float hi = (float)x;
      outff[(slot * NF + fn) * NV + v] = make_float2(hi, (float)(x - (double)hi));
    }
  }
}

// IndicatorMax (indicators_2d.jl / indicators_3d.jl:239-259): the maximum of
// the indicator variable over the nodes of each element, one warp per
// element, FP64 (float-float states read as hi + lo).
template <int D, typename S>
__global__ void indicator_max_kernel(const S* __restrict__ u, int64_t E, int NN, int variable,
                                     double gamma, double* __restrict__ out) {
  constexpr int NV = D + 2;
  const int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (e >= E) return;
  double m = -INFINITY;
  for (int n = lane; n < NN; n += 32) {
    double x[NV];
    const S* p = u + ((size_t)e * NN + n) * NV;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      if constexpr (std::is_same<S, double>::value)
        x[v] = p[v];
      else
        x[v] = (double)p[v].x + (double)p[v].y;
    }
    m = fmax(m, variable == 1 ? x[0] : Euler<D, double>::density_pressure(x, gamma));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) out[e] = m;
}

// Solution transfer of AMR (refine_element! / coarsen_elements!,
// amr_dg2d.jl:224-294, 429-485; amr_dg3d.jl): one thread per node of the
// adapted mesh.  mats: forward lower, upper, reverse lower, upper
// (row-major, M[a * N + b] = M[a, b]); the matrix along axis d of child q is
// the upper one when bit d of q is set.  Interpolated and projected values
// are formed in FP64 (float-float states: from hi + lo).
struct AdaptMats {
  double m[4][MAXN * MAXN];
};

template <int D, typename S>
__global__ void adapt_state_kernel(const S* __restrict__ uo, S* __restrict__ un,
                                   const int64_t* __restrict__ source, const int8_t* __restrict__ kind,
                                   int64_t E, int N, const AdaptMats M) {
  constexpr int NV = D + 2;
  const int NN = D == 2 ? N * N : N * N * N;
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E * NN) return;
  const int64_t e = k / NN;
  const int node = (int)(k - e * NN);
  const int kd = kind[e];
  const int64_t s0 = source[e];
  if (kd == 0) {
#pragma unroll
    for (int v = 0; v < NV; ++v) un[k * NV + v] = uo[(s0 * NN + node) * NV + v];
    return;
  }
  const int i[3] = {node % N, (node / N) % N, node / (N * N)};
  double acc[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
  const int nsrc = kd > 0 ? 1 : (1 << D);
  for (int q = 0; q < nsrc; ++q) {
    const int child = kd > 0 ? kd - 1 : q;
    const int64_t se = kd > 0 ? s0 : s0 + q;
    const double* Md[3];
#pragma unroll
    for (int d = 0; d < D; ++d) Md[d] = M.m[(kd > 0 ? 0 : 2) + ((child >> d) & 1)];
    for (int sn = 0; sn < NN; ++sn) {
      const int kk[3] = {sn % N, (sn / N) % N, sn / (N * N)};
      double w = 1.0;
#pragma unroll
      for (int d = 0; d < D; ++d) w *= Md[d][i[d] * N + kk[d]];
      const S* p = uo + (se * NN + sn) * NV;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double x;
        if constexpr (std::is_same<S, double>::value)
          x = p[v];
        else
          x = (double)p[v].x + (double)p[v].y;
        acc[v] += w * x;
      }
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    if constexpr (std::is_same<S, double>::value) {
      un[k * NV + v] = acc[v];
    } else {
      const float hi = (float)acc[v];
      un[k * NV + v] = make_float2(hi, (float)(acc[v] - (double)hi));
    }
  }
}

// out = a x + b y (y == nullptr: out = a x), elementwise; out may alias x or y.
__global__ void lincomb_kernel(int64_t n, double* out, double a, const double* x, double b,
                               const double* y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = y ? fma(b, y[i], a * x[i]) : a * x[i];
}

// apply_smoothing! as a gather (indicators_2d.jl:104-136): alpha_e =
// max(raw_e, 0.5 * raw_n for every element n across a face or a mortar).
template <typename R, typename O = double>
__global__ void smooth_alpha_kernel(const R* __restrict__ raw, const int32_t* __restrict__ nbr,
                                    int64_t E, int nfaces, int smooth, int32_t nbc,
                                    const int32_t* __restrict__ mnbr, O* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  R a = raw[e];
  if (smooth)
    for (int f = 0; f < nfaces; ++f) a = smooth_over_face<R>(a, nbr[e * nfaces + f], raw, nbc, mnbr);
  out[e] = (O)a;
}

}  // namespace tg

using namespace tg;

struct tg_ctx {
  int D = 0, N = 0, NN = 0, NV = 0, vi = 0, epb = 0, device = 0;
  bool fp64 = true;
  int64_t E = 0, ndofs = 0, nvalues = 0;
  DgParams P{};
  MixedParams MP{};
  cudaStream_t stream = nullptr;
  // state: FP64 values (fp64) or float-float pairs (mixed), 8 bytes per value
  void* d_u[2] = {nullptr, nullptr};
  int cur = 0;
  void* d_utmp = nullptr;            // double (fp64) or float (mixed)
  double* d_du = nullptr;            // tg_rhs_host scratch
  double* d_uscratch = nullptr;      // tg_rhs_host scratch
  double* d_stage64 = nullptr;       // mixed: FP64 staging of the state
  float2* d_uff = nullptr;           // mixed: float-float copy of a tg_rhs input
  void* d_alpha_raw = nullptr;
  double* d_alpha = nullptr;
  float* d_alpha_sm = nullptr;        // mixed 2D HG: smoothed blending factors (padded)
  // mixed 2D HG: rho*p of every node of the state d_u[cur], written by the
  // stage kernel that produced it (rp_valid), read by the next indicator
  float* d_rp = nullptr;
  bool rp_valid = false;
  // the clock's speed_bits hold the CFL reduction of the current state, made
  // when it was imported (to_ff_rp_speed_kernel); cleared by anything else
  // that sets the state
  bool speed_fresh = false;
  // host transfers that overlap the stepping (tg_prefetch_state, tg_fetch_state):
  // copy streams (0: host to device, 1: device to host), FP64 staging slots
  // and the events that order them with the context stream
  cudaStream_t xstream[2] = {nullptr, nullptr};
  double* d_xin[2] = {nullptr, nullptr};
  double* d_xout[2] = {nullptr, nullptr};
  cudaEvent_t ev_in_copied[2] = {nullptr, nullptr}, ev_in_used[2] = {nullptr, nullptr};
  cudaEvent_t ev_out_ready[2] = {nullptr, nullptr}, ev_out_done[2] = {nullptr, nullptr};
  bool in_pending[2] = {false, false}, in_used_rec[2] = {false, false};
  bool out_done_rec[2] = {false, false};
  // page-locked, device-mapped copy of the clock that tg_step polls: written by
  // a kernel, so the poll does not queue behind copies on the copy engines
  Clock* h_clock = nullptr;
  Clock* h_clock_dev = nullptr;
  // the clock's step count as of the end of the last tg_step (or 0 after it
  // was initialised), when nothing else has stepped the context since
  int64_t host_steps = 0;
  bool host_steps_valid = false;
  // buffers taken from the device's context pool (returned to it, in stream
  // order, when the context is destroyed)
  std::vector<void*> pool_ptrs;
  int32_t* d_nbr = nullptr;
  double* d_invj = nullptr;
  double* d_xline = nullptr;
  float* d_invj_f = nullptr;
  float* d_xline_f = nullptr;
  float4* d_sc0 = nullptr;            // mixed source phase of each element's first node
  float4* d_scn = nullptr;            // and of the node offsets (one table)
  int64_t nbound = 0;                 // boundary faces (non-periodic meshes)
  int32_t* d_bface = nullptr;         // [nbound][2]: element, direction
  float2* d_ghost = nullptr;          // mixed: [nbound + nmface][NF][NV] pre-pass output
  int64_t nmortar = 0;                // L2 mortars
  int64_t nmface = 0;                 // mortar face slots (2^(D-1) + 1 per mortar)
  int32_t* d_mtab = nullptr;          // [nmortar][2^(D-1) + 3]: elements, large side, orientation
  int32_t* d_mnbr = nullptr;          // [nmface][4]: elements across each mortar face
  double* d_mmat = nullptr;           // forward lower/upper, reverse lower/upper (row-major)
  float* d_mmat32 = nullptr;          // the same in FP32 (mixed pre-pass)
  double* d_mflux = nullptr;          // fp64: [nmface][NF][NV] mortar pre-pass output
  int8_t* d_scls = nullptr;           // mixed: size class of each element (source tables)
  double* d_amr_raw = nullptr;        // AMR indicator (unsmoothed, smoothed)
  double* d_amr_alpha = nullptr;
  int64_t* d_amap = nullptr;          // AMR transfer map of the last tg_adapt_state
  int8_t* d_akind = nullptr;
  double* d_weights = nullptr;
  // curvilinear meshes (mesh_type TG_MESH_CURVED)
  bool curved = false;
  tg::CurvedParams CP{};
  double* d_cmet = nullptr;           // [E][NN][5]: Ja^1, Ja^2, inverse Jacobian
  double2* d_csnv = nullptr;          // HG: subcell normals [E][2][N][N - 1]
  float2* d_csnv32 = nullptr;         // mixed HG: their FP32 copy
  double* d_csnv3 = nullptr;          // 3D HG: [E][3][N^2][N - 1] triples
  float4* d_csnv3_32 = nullptr;       // mixed 3D HG: (x, y, z, 0)
  float4* d_cja32 = nullptr;          // mixed: [E][NN] Ja^1, Ja^2
  float* d_cinvj32 = nullptr;         // mixed: [E][NN] inverse Jacobian
  double* d_cxy = nullptr;            // fp64 sources: [E][NN][2] node coordinates
  float4* d_csc = nullptr;            // mixed sources: [E][NN] sin/cos(pi (x + y))
  double* d_partial = nullptr;
  double* d_enorm = nullptr;          // error norms: per-element sums and maxima [E][2 nvar]
  double total_volume = 0.0;          // sum of the element volumes (TreeMesh: length_level_0^d)
  double* d_sums = nullptr;
  Clock* d_clock = nullptr;
  int32_t* d_status = nullptr;
  unsigned long long* d_speed = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  bool clock_valid = false;
  bool uploaded = false;
  tg_mlp* learned = nullptr;      // learned shock indicator (HG contexts), or null
  const void* view_state = nullptr;  // state the learned indicator reads next
  std::vector<double> weights;
  std::vector<double*> vectors;      // tg_vector_create allocations (freed with the context)
  std::string err;
};

static thread_local std::string g_create_err;

namespace tg {
void set_thread_error(const char* msg) { g_create_err = msg; }
int mlp_alpha(tg_mlp* m, tg_ctx* c, void* alpha_raw, bool fp64, float alpha_min, float alpha_max);
}  // namespace tg

static int fail(tg_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c)
    c->err = buf;
  else
    g_create_err = buf;
  return code;
}

#define CUDA_TRY(ctx, call)                                                                    \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail((ctx), TG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));         \
  } while (0)

static size_t rsize(const tg_ctx* c) { return c->fp64 ? sizeof(double) : sizeof(float); }
// Padding (elements) of per-element FP32 arrays that bulk copies read in
// 16-byte groups past the last element.
constexpr int64_t kElemPad = 64;

// Per-device memory pool for the buffers of contexts: an AMR pass destroys a
// context and creates one for the adapted mesh, so their buffers come from a
// pool that keeps up to 4 GiB of freed memory (its release threshold) instead
// of cudaMalloc / cudaFree every time; freed memory above that goes back to
// the device at the next synchronisation, for other allocators to use.
static cudaMemPool_t context_pool(int device) {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  if (device < 0 || device >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!pools[device]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = 4ull << 30;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[device] = p;
  }
  return pools[device];
}

static void free_ctx(tg_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  for (int p = 0; p < 2; ++p)
    if (c->graph[p]) cudaGraphExecDestroy(c->graph[p]);
  void* ptrs[] = {c->d_u[0], c->d_u[1], c->d_utmp, c->d_du, c->d_uscratch, c->d_stage64,
                  c->d_uff, c->d_alpha_raw, c->d_alpha, c->d_alpha_sm, c->d_rp, c->d_nbr, c->d_invj, c->d_xline,
                  c->d_invj_f, c->d_xline_f, c->d_sc0, c->d_scn, c->d_bface, c->d_ghost, c->d_mtab, c->d_mnbr, c->d_mmat, c->d_mmat32, c->d_mflux, c->d_scls, c->d_amr_raw, c->d_amr_alpha, c->d_amap, c->d_akind, c->d_weights, c->d_cmet, c->d_csnv, c->d_csnv32, c->d_csnv3, c->d_csnv3_32, c->d_cja32, c->d_cinvj32, c->d_cxy, c->d_csc, c->d_partial, c->d_enorm, c->d_sums, c->d_clock,
                  c->d_status, c->d_speed};
  for (int k = 0; k < 2; ++k)
    if (c->xstream[k]) cudaStreamSynchronize(c->xstream[k]);
  for (void* p : ptrs)
    if (p && std::find(c->pool_ptrs.begin(), c->pool_ptrs.end(), p) == c->pool_ptrs.end())
      cudaFree(p);
  // cudaFree waits for the whole device; the pool frees keep that guarantee
  // (work on other streams that still reads a buffer ends before its reuse)
  if (!c->pool_ptrs.empty()) cudaDeviceSynchronize();
  for (void* p : c->pool_ptrs) cudaFreeAsync(p, c->stream);
  for (int k = 0; k < 2; ++k) {
    if (c->d_xin[k]) cudaFree(c->d_xin[k]);
    if (c->d_xout[k]) cudaFree(c->d_xout[k]);
    for (cudaEvent_t ev : {c->ev_in_copied[k], c->ev_in_used[k], c->ev_out_ready[k], c->ev_out_done[k]})
      if (ev) cudaEventDestroy(ev);
    if (c->xstream[k]) cudaStreamDestroy(c->xstream[k]);
  }
  for (double* p : c->vectors) cudaFree(p);
  if (c->h_clock) cudaFreeHost(c->h_clock);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

static unsigned conv_blocks(int64_t n) {
  return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
}

static int ensure(tg_ctx* c, void** p, size_t bytes) {
  if (!*p) CUDA_TRY(c, cudaMalloc(p, bytes));
  return TG_OK;
}

// FP64 state (Trixi layout) -> context representation in `dst`.  Into the
// current state of a context that keeps the indicator input (mixed 2D shock
// capturing), the same pass writes rho*p of every node (rp_valid).
static int import_state(tg_ctx* c, const double* src, void* dst) {
  if (c->fp64) {
    if (src != dst)
      CUDA_TRY(c, cudaMemcpyAsync(dst, src, sizeof(double) * c->nvalues, cudaMemcpyDeviceToDevice,
                                  c->stream));
    return TG_OK;
  }
  c->speed_fresh = false;
  if (c->d_rp && dst == c->d_u[c->cur] && c->NV == 4) {
    if (!c->curved && c->NN == 16) {
      // the CFL reduction of the new state in the same pass (ctx_clock_prepare
      // then skips its own)
      speed_reset_kernel<<<1, 1, 0, c->stream>>>(&c->d_clock->speed_bits);
      if (((uintptr_t)src & 15) == 0)
        to_ff_rp_speed_pair_kernel<<<conv_blocks(2 * c->ndofs), 256, 0, c->stream>>>(
            (const double2*)src, (float4*)dst, c->ndofs, c->MP.gamma, c->d_rp,
            (float)c->P.gamma, c->d_invj_f, &c->d_clock->speed_bits, c->d_status);
      else
        to_ff_rp_speed_kernel<16><<<conv_blocks(c->ndofs), 256, 0, c->stream>>>(
            src, (float2*)dst, c->ndofs, c->MP.gamma, c->d_rp, (float)c->P.gamma, c->d_invj_f,
            &c->d_clock->speed_bits, c->d_status);
      CUDA_TRY(c, cudaGetLastError());
      c->speed_fresh = true;
    } else {
      to_ff_rp_kernel<<<conv_blocks(c->ndofs), 256, 0, c->stream>>>(src, (float2*)dst, c->ndofs,
                                                                     c->MP.gamma, c->d_rp);
      CUDA_TRY(c, cudaGetLastError());
    }
    c->rp_valid = true;
    return TG_OK;
  }
  if (((uintptr_t)src & 15) == 0 && c->nvalues % 2 == 0)
    to_ff2_kernel<<<conv_blocks(c->nvalues / 2), 256, 0, c->stream>>>(
        (const double2*)src, (float4*)dst, c->nvalues / 2);
  else
    to_ff_kernel<<<conv_blocks(c->nvalues), 256, 0, c->stream>>>(src, (float2*)dst, c->nvalues);
  CUDA_TRY(c, cudaGetLastError());
  if (dst == c->d_u[c->cur]) c->rp_valid = false;
  return TG_OK;
}

// Float-float state -> FP64 values in `out` (device or mapped host memory):
// 16-byte accesses when `out` allows them.
static void launch_from_ff(tg_ctx* c, const void* in, double* out) {
  if (((uintptr_t)out & 15) == 0 && c->nvalues % 2 == 0)
    from_ff2_kernel<<<conv_blocks(c->nvalues / 2), 256, 0, c->stream>>>(
        (const float4*)in, (double2*)out, c->nvalues / 2);
  else
    from_ff_kernel<<<conv_blocks(c->nvalues), 256, 0, c->stream>>>((const float2*)in, out,
                                                                    c->nvalues);
}

// Context state -> FP64 values (for mixed: into d_stage64); returns the FP64 pointer.
static const double* export_state(tg_ctx* c, int* rc) {
  *rc = TG_OK;
  if (c->fp64) return (const double*)c->d_u[c->cur];
  if ((*rc = ensure(c, (void**)&c->d_stage64, sizeof(double) * c->nvalues))) return nullptr;
  launch_from_ff(c, c->d_u[c->cur], c->d_stage64);
  if (cudaGetLastError() != cudaSuccess) {
    *rc = fail(c, TG_ERR_CUDA, "state conversion launch failed");
    return nullptr;
  }
  return c->d_stage64;
}

namespace tg {
const float* ctx_state_rho_p(tg_ctx* c);
}

// Mixed 2D TreeMesh contexts without mortars: the persistent stage kernel
// applies apply_smoothing! to the raw factors itself (MixedArgs::alpha_gather),
// so no smoothing pass runs between the indicator and the stage kernel.
static bool alpha_gather_mode(const tg_ctx* c) {
  return !c->fp64 && !c->curved && c->D == 2 && c->nmortar == 0;
}

// Blending factors of a state in the context representation: the HG (or
// learned) indicator, unsmoothed, into d_alpha_raw; for mixed 2D TreeMesh
// contexts with mortars also apply_smoothing! into d_alpha_sm, which the
// persistent stage kernel copies with the element block (the other kernels
// smooth inline).
static int indicator(tg_ctx* c, const void* u) {
  if (c->vi != VI_HG) return TG_OK;
  int rc;
  if (c->learned) {
    c->view_state = u;
    rc = mlp_alpha(c->learned, c, c->d_alpha_raw, c->fp64, (float)c->P.alpha_min,
                   (float)c->P.alpha_max);
    c->view_state = nullptr;
    if (rc) return rc;
  } else {
    const float* rp = u == c->d_u[c->cur] ? tg::ctx_state_rho_p(c) : nullptr;
    if (c->fp64)
      rc = launch_indicator(c->D, c->N, true, c->P, (const double*)u, c->d_alpha_raw, c->stream);
    else if (rp)
      rc = launch_hg_alpha_rp(c->N, c->MP, rp, (float*)c->d_alpha_raw, c->stream);
    else if (c->D == 2)
      rc = launch_indicator_mixed_2(c->N, c->MP, (const float2*)u, (float*)c->d_alpha_raw,
                                    c->stream);
    else
      rc = launch_indicator_mixed_3(c->N, c->MP, (const float2*)u, (float*)c->d_alpha_raw,
                                    c->stream);
    if (rc != 0) return fail(c, TG_ERR_CUDA, "indicator kernel launch failed (%d)", rc);
  }
  if (!c->fp64 && !c->curved && c->D == 2 && !alpha_gather_mode(c)) {
    smooth_alpha_kernel<float, float><<<(unsigned)((c->E + 255) / 256), 256, 0, c->stream>>>(
        (const float*)c->d_alpha_raw, c->d_nbr, c->E, 2 * c->D, c->P.alpha_smooth, c->P.nbc,
        c->d_mnbr, c->d_alpha_sm);
    CUDA_TRY(c, cudaGetLastError());
  }
  return TG_OK;
}

// Mortar pre-pass for the state u_in (context representation).
static void launch_mortars(tg_ctx* c, const void* u_in) {
  const unsigned nb = (unsigned)c->nmortar;
  if (c->fp64) {
    if (c->D == 2)
      mortar_flux_kernel<2, double><<<nb, 128, 0, c->stream>>>(
          c->P, (const double*)u_in, c->d_mtab, c->d_mmat, c->nmortar, c->N, 0, c->d_mflux, nullptr);
    else
      mortar_flux_kernel<3, double><<<nb, 128, 0, c->stream>>>(
          c->P, (const double*)u_in, c->d_mtab, c->d_mmat, c->nmortar, c->N, 0, c->d_mflux, nullptr);
  } else {
    if (c->D == 2)
      mortar_flux_ff_kernel<2><<<nb, 128, 0, c->stream>>>(c->MP, (const float2*)u_in, c->d_mtab,
                                                          c->d_mmat32, c->nmortar, c->N, c->nbound,
                                                          c->d_ghost);
    else
      mortar_flux_ff_kernel<3><<<nb, 128, 0, c->stream>>>(c->MP, (const float2*)u_in, c->d_mtab,
                                                          c->d_mmat32, c->nmortar, c->N, c->nbound,
                                                          c->d_ghost);
  }
}

// One element-kernel launch.  u_in is in the context representation.
static int launch_kernel(tg_ctx* c, int mode, const void* u_in, void* u_out, double* du_out,
                         double t_rhs, int stage, bool reduce, bool write_rp = false) {
  int rc;
  c->speed_fresh = false;
  if (c->nmortar > 0) launch_mortars(c, u_in);
  if (c->curved) {
    StageArgs A{};
    MixedArgs M{};
    A.status = M.status = c->d_status;
    A.clock = M.clock = c->d_clock;
    A.mode = M.mode = mode;
    A.u_in = (const double*)u_in;
    A.u_out = (double*)u_out;
    M.u_in = (const float2*)u_in;
    M.u_out = (float2*)u_out;
    A.du_out = M.du_out = du_out;
    A.u_tmp = c->d_utmp;
    M.u_tmp = (float*)c->d_utmp;
    A.t_rhs = M.t_rhs = t_rhs;
    A.alpha_raw = c->d_alpha_raw;
    M.alpha_raw = (const float*)c->d_alpha_raw;
    if (mode == MODE_STAGE) {
      A.a = M.a = CK_A[stage];
      A.b = M.b = CK_B[stage];
      A.c = M.c = CK_C[stage];
      A.zero_tmp = M.zero_tmp = stage == 0;
      M.stage = stage;
    } else {
      const double sn = std::sin(M_PI * t_rhs), cs = std::cos(M_PI * t_rhs);
      M.sin_t = (float)sn;
      M.cos_t = (float)cs;
      M.sin_tl = (float)(sn - (double)M.sin_t);
      M.cos_tl = (float)(cs - (double)M.cos_t);
    }
    A.speed_bits = M.speed_bits = reduce ? &c->d_clock->speed_bits : nullptr;
    if (c->D == 3) {
      if (tg::launch_curved3(c->CP, c->fp64 ? &A : nullptr, c->fp64 ? nullptr : &M, c->stream) != 0)
        return fail(c, TG_ERR_CUDA, "curvilinear 3D kernel launch failed: %s",
                    cudaGetErrorString(cudaGetLastError()));
      return TG_OK;
    }
    if (!c->fp64 && c->nbound > 0 &&
        tg::launch_curved_ghost(c->CP, c->nbound, c->d_clock,
                                mode == MODE_STAGE ? CK_C[stage] : 0.0, t_rhs, mode, c->d_ghost,
                                c->stream) != 0)
      return fail(c, TG_ERR_CUDA, "curvilinear boundary pre-pass launch failed");
    rc = tg::launch_curved(c->CP, c->fp64 ? &A : nullptr, c->fp64 ? nullptr : &M, c->stream);
    if (rc != 0) {
      cudaError_t e = cudaGetLastError();
      return fail(c, TG_ERR_CUDA, "curvilinear kernel launch failed (%d): %s", rc,
                  cudaGetErrorString(e));
    }
    return TG_OK;
  }
  if (c->fp64) {
    StageArgs A{};
    A.alpha_raw = c->d_alpha_raw;
    A.status = c->d_status;
    A.clock = c->d_clock;
    A.mode = mode;
    A.u_in = (const double*)u_in;
    A.u_out = (double*)u_out;
    A.du_out = du_out;
    A.u_tmp = c->d_utmp;
    A.t_rhs = t_rhs;
    if (mode == MODE_STAGE) {
      A.a = CK_A[stage];
      A.b = CK_B[stage];
      A.c = CK_C[stage];
      A.zero_tmp = stage == 0;
    }
    A.speed_bits = reduce ? &c->d_clock->speed_bits : nullptr;
    rc = launch_element(c->D, c->N, true, c->vi, c->epb, c->P, A, c->stream);
  } else {
    MixedArgs A{};
    A.alpha_raw = (const float*)c->d_alpha_raw;
    if (alpha_gather_mode(c)) {
      A.alpha_smoothed = (const float*)c->d_alpha_raw;
      A.alpha_gather = c->P.alpha_smooth ? 1 : 0;
    } else {
      A.alpha_smoothed = c->d_alpha_sm;
    }
    A.rp_out = write_rp && mode == MODE_STAGE ? c->d_rp : nullptr;
    A.status = c->d_status;
    A.clock = c->d_clock;
    A.mode = mode;
    A.u_in = (const float2*)u_in;
    A.u_out = (float2*)u_out;
    A.du_out = du_out;
    A.u_tmp = (float*)c->d_utmp;
    A.t_rhs = t_rhs;
    if (mode == MODE_STAGE) {
      A.a = CK_A[stage];
      A.b = CK_B[stage];
      A.c = CK_C[stage];
      A.zero_tmp = stage == 0;
      A.stage = stage;
    } else {
      const double sn = std::sin(M_PI * t_rhs), cs = std::cos(M_PI * t_rhs);
      A.sin_t = (float)sn;
      A.cos_t = (float)cs;
      A.sin_tl = (float)(sn - (double)A.sin_t);
      A.cos_tl = (float)(cs - (double)A.cos_t);
    }
    A.speed_bits = reduce ? &c->d_clock->speed_bits : nullptr;
    if (c->nbound > 0) {
      // boundary pre-pass for this stage's input state
      const int64_t nk = c->nbound * (c->NN / c->N);
      const unsigned nb = (unsigned)((nk + 127) / 128);
      const double cs = mode == MODE_STAGE ? CK_C[stage] : 0.0;
      if (c->D == 2)
        boundary_ghost_kernel<2><<<nb, 128, 0, c->stream>>>(c->P, (const float2*)u_in, c->d_bface,
                                                            c->nbound, c->N, c->d_clock, cs, t_rhs,
                                                            mode, c->d_ghost);
      else
        boundary_ghost_kernel<3><<<nb, 128, 0, c->stream>>>(c->P, (const float2*)u_in, c->d_bface,
                                                            c->nbound, c->N, c->d_clock, cs, t_rhs,
                                                            mode, c->d_ghost);
    }
    rc = launch_mixed(c->D, c->N, c->vi, c->epb, c->MP, A, c->stream);
  }
  if (rc != 0) {
    cudaError_t e = cudaGetLastError();
    return fail(c, TG_ERR_CUDA, "element kernel launch failed (%d): %s", rc, cudaGetErrorString(e));
  }
  return TG_OK;
}

// Enqueue one fused 2N stage reading d_u[cur] and writing d_u[cur ^ 1].
static int enqueue_stage(tg_ctx* c, int stage, bool reduce_speed) {
  int rc = indicator(c, c->d_u[c->cur]);
  if (rc) return rc;
  rc = launch_kernel(c, MODE_STAGE, c->d_u[c->cur], c->d_u[c->cur ^ 1], nullptr, 0.0, stage,
                     reduce_speed, true);
  if (rc) return rc;
  c->cur ^= 1;
  c->rp_valid = c->d_rp != nullptr;  // the kernel wrote rho*p of its output
  return TG_OK;
}

// rho*p of the current state into d_rp (before a step graph whose first
// indicator reads it, after the state was set from outside the stage kernels).
static int refresh_rho_p(tg_ctx* c) {
  if (!c->d_rp || c->rp_valid) return TG_OK;
  rho_p_ff_kernel<<<conv_blocks(c->ndofs), 256, 0, c->stream>>>(
      (const float2*)c->d_u[c->cur], c->ndofs, c->NV, c->MP.gamma, c->d_rp);
  CUDA_TRY(c, cudaGetLastError());
  c->rp_valid = true;
  return TG_OK;
}

// CFL reduction of a state: FP64 values, or (ff) the float-float state of a
// mixed context in that context's FP32 wave-speed arithmetic.
static int reduce_speed(tg_ctx* c, const void* u, bool ff, unsigned long long* dst) {
  speed_reset_kernel<<<1, 1, 0, c->stream>>>(dst);
  if (c->curved) {
    const int rc = c->D == 3 ? tg::launch_curved3_speed(c->CP, u, ff, dst, c->d_status, c->stream)
                             : tg::launch_curved_speed(c->CP, u, ff, dst, c->d_status, c->stream);
    if (rc != 0) return fail(c, TG_ERR_CUDA, "curvilinear wave-speed launch failed");
    return TG_OK;
  }
  // warps stride over the elements: at most 16 blocks of 4 warps per SM
  const unsigned nb = (unsigned)std::min<int64_t>((c->E + 3) / 4, 152 * 16);
  if (c->D == 2) {
    if (ff)
      max_speed_ff_kernel<2><<<nb, 128, 0, c->stream>>>((const float2*)u, c->d_invj_f, c->E, c->NN,
                                                       (float)c->P.gamma, dst, c->d_status);
    else
      max_speed_kernel<2, double><<<nb, 128, 0, c->stream>>>((const double*)u, c->d_invj, c->E,
                                                            c->NN, c->P.gamma, dst, c->d_status);
  } else {
    if (ff)
      max_speed_ff_kernel<3><<<nb, 128, 0, c->stream>>>((const float2*)u, c->d_invj_f, c->E, c->NN,
                                                       (float)c->P.gamma, dst, c->d_status);
    else
      max_speed_kernel<3, double><<<nb, 128, 0, c->stream>>>((const double*)u, c->d_invj, c->E,
                                                            c->NN, c->P.gamma, dst, c->d_status);
  }
  CUDA_TRY(c, cudaGetLastError());
  return TG_OK;
}

// Metric terms and source tables of a curvilinear context, and its kernel
// parameters (after the generic setup of tg_ctx_create).
static int curved_setup(tg_ctx* c, const tg_config* cfg) {
  const int N = c->N, NN = c->NN, D = c->D;
  const int64_t E = c->E;
  const size_t nq = (size_t)E * NN;
  const int MS = D * D + 1;  // metric values per node: Ja^d_c (d-major), inverse Jacobian
  std::vector<double> met(nq * MS);
  for (size_t k = 0; k < nq; ++k) {
    for (int m = 0; m < D * D; ++m) met[k * MS + m] = cfg->contravariant_vectors[k * D * D + m];
    met[k * MS + D * D] = cfg->inverse_jacobian[k];
  }
  CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_cmet, sizeof(double) * met.size()));
  CUDA_TRY(nullptr, cudaMemcpy(c->d_cmet, met.data(), sizeof(double) * met.size(),
                               cudaMemcpyHostToDevice));
  const bool src = c->P.source == SRC_CONVERGENCE_TEST;
  if (!c->fp64 && D == 3) {
    // per node three float4 {Ja^d_x, Ja^d_y, Ja^d_z, (d = 0: inverse Jacobian)}
    std::vector<float4> ja(nq * 3);
    for (size_t k = 0; k < nq; ++k) {
      const double* m = &met[k * MS];
      for (int d = 0; d < 3; ++d)
        ja[k * 3 + d] = make_float4((float)m[3 * d], (float)m[3 * d + 1], (float)m[3 * d + 2],
                                    d == 0 ? (float)m[9] : 0.0f);
    }
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_cja32, sizeof(float4) * nq * 3));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_cja32, ja.data(), sizeof(float4) * nq * 3,
                                 cudaMemcpyHostToDevice));
  } else if (!c->fp64) {
    std::vector<float4> ja(nq);
    std::vector<float> ij(nq);
    for (size_t k = 0; k < nq; ++k) {
      const double* m = &met[k * 5];
      ja[k] = make_float4((float)m[0], (float)m[1], (float)m[2], (float)m[3]);
      ij[k] = (float)m[4];
    }
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_cja32, sizeof(float4) * nq));
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_cinvj32, sizeof(float) * nq));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_cja32, ja.data(), sizeof(float4) * nq,
                                 cudaMemcpyHostToDevice));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_cinvj32, ij.data(), sizeof(float) * nq,
                                 cudaMemcpyHostToDevice));
  }
  if (!c->fp64) {
    if (src) {
      // sin/cos(pi (x + y (+ z))) per node as float-float pairs; the stage
      // kernel combines them with sin/cos(pi t) by the angle-difference formula
      std::vector<float4> sc(nq);
      for (size_t k = 0; k < nq; ++k) {
        double ph = 0.0;
        for (int d = 0; d < D; ++d) ph += cfg->node_coordinates[k * D + d];
        const double sn = std::sin(M_PI * ph), cs = std::cos(M_PI * ph);
        const float sh = (float)sn, ch = (float)cs;
        sc[k] = make_float4(sh, ch, (float)(sn - (double)sh), (float)(cs - (double)ch));
      }
      CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_csc, sizeof(float4) * nq));
      CUDA_TRY(nullptr, cudaMemcpy(c->d_csc, sc.data(), sizeof(float4) * nq,
                                   cudaMemcpyHostToDevice));
    }
  }
  if ((src && c->fp64) || c->nbound > 0) {
    // FP64 node coordinates: sources of FP64 contexts, Dirichlet boundary values
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_cxy, sizeof(double) * nq * D));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_cxy, cfg->node_coordinates, sizeof(double) * nq * D,
                                 cudaMemcpyHostToDevice));
  }
  if (c->vi == VI_HG && D == 3) {
    // calc_normalvectors_subcell_fv! (dgsem_structured/containers_3d.jl:352-470):
    // per direction d, Ja^d at the line's first node plus the partial sums of
    // w_m D[m, :] Ja^d along the line (D by barycentric weights, as in 2D)
    const double* x = cfg->nodes;
    std::vector<double> wb(N, 1.0), Dm((size_t)N * N, 0.0);
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < N; ++k)
        if (k != j) wb[j] /= x[j] - x[k];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        if (j != i) {
          Dm[i * N + j] = (wb[j] / wb[i]) / (x[i] - x[j]);
          Dm[i * N + i] -= Dm[i * N + j];
        }
    const int NF = N * N;
    const size_t nsv = (size_t)E * 3 * NF * (N - 1);
    std::vector<double> snv(nsv * 3);
    for (int64_t e = 0; e < E; ++e)
      for (int dd = 0; dd < 3; ++dd)
        for (int l = 0; l < NF; ++l) {
          const int l0 = l % N, l1 = l / N;
          auto ja = [&](int a, int xyz) {
            const int q = dd == 0 ? a + N * (l0 + N * l1)
                                  : (dd == 1 ? l0 + N * (a + N * l1) : l0 + N * (l1 + N * a));
            return met[((size_t)e * NN + q) * MS + 3 * dd + xyz];
          };
          double acc[3] = {ja(0, 0), ja(0, 1), ja(0, 2)};
          for (int i = 0; i < N - 1; ++i) {
            for (int m = 0; m < N; ++m) {
              const double wd = cfg->weights[i] * Dm[i * N + m];
              for (int xyz = 0; xyz < 3; ++xyz) acc[xyz] += wd * ja(m, xyz);
            }
            for (int xyz = 0; xyz < 3; ++xyz)
              snv[((((size_t)e * 3 + dd) * NF + l) * (N - 1) + i) * 3 + xyz] = acc[xyz];
          }
        }
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_csnv3, sizeof(double) * snv.size()));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_csnv3, snv.data(), sizeof(double) * snv.size(),
                                 cudaMemcpyHostToDevice));
    if (!c->fp64) {
      std::vector<float4> s32(nsv);
      for (size_t k = 0; k < nsv; ++k)
        s32[k] = make_float4((float)snv[3 * k], (float)snv[3 * k + 1], (float)snv[3 * k + 2], 0.0f);
      CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_csnv3_32, sizeof(float4) * nsv));
      CUDA_TRY(nullptr, cudaMemcpy(c->d_csnv3_32, s32.data(), sizeof(float4) * nsv,
                                   cudaMemcpyHostToDevice));
    }
  }
  if (c->vi == VI_HG && D == 2) {
    // calc_normalvectors_subcell_fv! (dgsem_structured/containers_2d.jl:200-298):
    // the normal of the subcell interface between nodes i and i + 1 of a line
    // is Ja at the line's first node plus the partial sums of w_m D[m, :] Ja
    // along the line (D: polynomial_derivative_matrix by barycentric weights,
    // Kopriva, Implementing Spectral Methods, algorithm 37)
    const double* x = cfg->nodes;
    std::vector<double> wb(N, 1.0), Dm((size_t)N * N, 0.0);
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < N; ++k)
        if (k != j) wb[j] /= x[j] - x[k];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        if (j != i) {
          Dm[i * N + j] = (wb[j] / wb[i]) / (x[i] - x[j]);
          Dm[i * N + i] -= Dm[i * N + j];
        }
    const size_t nsv = (size_t)E * 2 * N * (N - 1);
    std::vector<double2> snv(nsv);
    for (int64_t e = 0; e < E; ++e)
      for (int dd = 0; dd < 2; ++dd)
        for (int l = 0; l < N; ++l) {
          auto ja = [&](int a, int xy) {
            const int q = dd == 0 ? a + N * l : l + N * a;
            return met[((size_t)e * NN + q) * MS + 2 * dd + xy];
          };
          double acc[2] = {ja(0, 0), ja(0, 1)};
          for (int i = 0; i < N - 1; ++i) {
            for (int m = 0; m < N; ++m) {
              const double wd = cfg->weights[i] * Dm[i * N + m];
              for (int xy = 0; xy < 2; ++xy) acc[xy] += wd * ja(m, xy);
            }
            snv[(((size_t)e * 2 + dd) * N + l) * (N - 1) + i] = make_double2(acc[0], acc[1]);
          }
        }
    CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_csnv, sizeof(double2) * nsv));
    CUDA_TRY(nullptr, cudaMemcpy(c->d_csnv, snv.data(), sizeof(double2) * nsv,
                                 cudaMemcpyHostToDevice));
    if (!c->fp64) {
      std::vector<float2> snv32(nsv);
      for (size_t k = 0; k < nsv; ++k) snv32[k] = make_float2((float)snv[k].x, (float)snv[k].y);
      CUDA_TRY(nullptr, cudaMalloc((void**)&c->d_csnv32, sizeof(float2) * nsv));
      CUDA_TRY(nullptr, cudaMemcpy(c->d_csnv32, snv32.data(), sizeof(float2) * nsv,
                                   cudaMemcpyHostToDevice));
    }
  }
  tg::CurvedParams& C = c->CP;
  C.nelements = E;
  C.N = N;
  C.vi = c->vi;
  C.volume_flux = c->P.volume_flux;
  C.surface_flux = c->P.surface_flux;
  C.source = c->P.source;
  C.gamma = c->P.gamma;
  C.inv_gamma_minus_one = c->P.inv_gamma_minus_one;
  C.eos = c->MP.eos;
  for (int k = 0; k < MAXN * MAXN; ++k) {
    C.Dhat[k] = c->P.Dhat[k];
    C.Dsplit[k] = c->P.Dsplit[k];
    C.Dhat32[k] = (float)c->P.Dhat[k];
    C.Dsplit32[k] = (float)c->P.Dsplit[k];
  }
  for (int k = 0; k < MAXN; ++k) {
    C.inv_weights[k] = c->P.inv_weights[k];
    C.inv_weights32[k] = (float)c->P.inv_weights[k];
  }
  C.nbr = c->d_nbr;
  C.met = c->d_cmet;
  C.ja32 = c->d_cja32;
  C.invj32 = c->d_cinvj32;
  C.xy = c->d_cxy;
  C.sc = c->d_csc;
  C.bc_ic = c->P.bc_ic;
  for (int k = 0; k < 4; ++k) C.bc_par[k] = c->P.bc_par[k];
  C.bface = c->d_bface;
  C.ghost = c->d_ghost;
  C.fv_flux = c->P.fv_flux;
  C.alpha_smooth = c->P.alpha_smooth;
  C.alpha_atol = c->P.alpha_atol;
  C.snv = c->d_csnv;
  C.snv32 = c->d_csnv32;
  C.snv3 = c->d_csnv3;
  C.snv3_32 = c->d_csnv3_32;
  return TG_OK;
}

namespace tg {
// State, shape and basis of a context for the learned indicator (tg_learned.cu).
int ctx_state_view(tg_ctx* c, const void** state, int* is_ff, int* D, int* N, int64_t* E,
                   double* gamma, const double** vinv_rowmajor, void** stream) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  *state = c->view_state ? c->view_state : c->d_u[c->cur];
  *is_ff = c->fp64 ? 0 : 1;
  *D = c->D;
  *N = c->N;
  *E = c->E;
  *gamma = c->P.gamma;
  *vinv_rowmajor = c->P.Vinv;
  *stream = (void*)c->stream;
  return TG_OK;
}

int32_t* ctx_status_word(tg_ctx* c) { return c->d_status; }

// rho*p of the state the indicator is about to read, when the stage kernel
// that produced that state wrote it (mixed 2D shock-capturing contexts), else
// null
const float* ctx_state_rho_p(tg_ctx* c) {
  if (!c->d_rp || !c->rp_valid) return nullptr;
  if (c->view_state && c->view_state != c->d_u[c->cur]) return nullptr;
  return c->d_rp;
}

int ctx_set_alpha_source(tg_ctx* c, tg_mlp* m) {
  if (m && c->vi != VI_HG)
    return fail(c, TG_ERR_STATE, "the learned indicator replaces the HG indicator: "
                                 "VolumeIntegralShockCapturingHG contexts only");
  c->learned = m;
  // step graphs embed the indicator launches: capture them again
  for (int p = 0; p < 2; ++p)
    if (c->graph[p]) {
      cudaGraphExecDestroy(c->graph[p]);
      c->graph[p] = nullptr;
    }
  return TG_OK;
}
}  // namespace tg

extern "C" {

int tg_api_version(void) { return TG_API_VERSION; }

int tg_last_error(const tg_ctx* ctx, char* buf, size_t len) {
  if (!buf || len == 0) return TG_ERR_INVALID_ARGUMENT;
  const std::string& s = ctx ? ctx->err : g_create_err;
  const size_t n = std::min(len - 1, s.size());
  std::memcpy(buf, s.data(), n);
  buf[n] = 0;
  return TG_OK;
}

int tg_ctx_create(const tg_config* cfg, tg_ctx** out) {
  if (!cfg || !out) return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const int D = cfg->ndims;
  if (D != 2 && D != 3) return fail(nullptr, TG_ERR_UNSUPPORTED, "ndims must be 2 or 3");
  const int N = cfg->polydeg + 1;
  // (curvilinear meshes check their own kernels below)
  if (cfg->mesh_type != TG_MESH_CURVED && default_epb(D, N) == 0)
    return fail(nullptr, TG_ERR_UNSUPPORTED, "polydeg %d is not compiled for %dD", cfg->polydeg, D);
  if (cfg->nelements <= 0) return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "nelements must be > 0");
  if (cfg->ninterfaces < 0 || cfg->ninterfaces > (int64_t)D * cfg->nelements)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "more interfaces than element faces");
  if (cfg->volume_integral < 0 || cfg->volume_integral > 2)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "unknown volume integral %d", cfg->volume_integral);
  const int fl[3] = {cfg->volume_flux, cfg->surface_flux, cfg->volume_flux_fv};
  for (int k = 0; k < 3; ++k)
    if (fl[k] < 0 || fl[k] > 7) return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "unknown flux %d", fl[k]);
  if ((cfg->volume_flux == TG_FLUX_HLLC || cfg->volume_flux == TG_FLUX_HLLE) &&
      cfg->volume_integral != TG_VOLUME_WEAK_FORM)
    return fail(nullptr, TG_ERR_UNSUPPORTED,
                "flux_hllc / flux_hlle are surface fluxes: not two-point volume fluxes for flux "
                "differencing");
  if (cfg->source_terms != TG_SOURCE_NONE && cfg->source_terms != TG_SOURCE_CONVERGENCE_TEST)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "unknown source terms %d", cfg->source_terms);
  if (cfg->precision != TG_PRECISION_FP64 && cfg->precision != TG_PRECISION_MIXED)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "unknown precision %d", cfg->precision);
  if (!cfg->nodes || !cfg->weights || !cfg->inverse_weights || !cfg->derivative_hat ||
      !cfg->derivative_split || !cfg->inverse_vandermonde_legendre || !cfg->neighbor_ids ||
      !cfg->orientations || !cfg->inverse_jacobian)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "missing basis or mesh array");
  if (cfg->source_terms != TG_SOURCE_NONE && !cfg->node_coordinates)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "source terms need node_coordinates");
  const bool mixed = cfg->precision == TG_PRECISION_MIXED;
  if (cfg->mesh_type != TG_MESH_TREE && cfg->mesh_type != TG_MESH_CURVED)
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "unknown mesh type %d", cfg->mesh_type);
  const bool curved = cfg->mesh_type == TG_MESH_CURVED;
  if (curved) {
    // StructuredMesh / P4estMesh bricks: the curvilinear kernels of tg_curved.cu
    // (2D) and tg_curved3.cu (3D)
    // 3D: tg_curved3.cu is built for polydeg 3 and 5, weak form or flux differencing
    if (D == 2 ? tg::curved_epb(N) == 0 : !tg::curved3_supported(N))
      return fail(nullptr, TG_ERR_UNSUPPORTED, "curvilinear meshes: polydeg %d is not compiled",
                  cfg->polydeg);
    const bool hg = cfg->volume_integral == TG_VOLUME_SHOCK_CAPTURING_HG;
    if (hg && D == 3 && N != 4)
      return fail(nullptr, TG_ERR_UNSUPPORTED,
                  "3D curvilinear meshes: shock capturing at polydeg 3 only");
    const int vf = cfg->volume_flux, sf = cfg->surface_flux;
    if (hg && (cfg->volume_flux_fv == TG_FLUX_HLLC || cfg->volume_flux_fv == TG_FLUX_HLLE))
      return fail(nullptr, TG_ERR_UNSUPPORTED, "curvilinear meshes: FV flux_hllc / flux_hlle");
    if ((cfg->volume_integral == TG_VOLUME_FLUX_DIFFERENCING || hg) &&
        vf != TG_FLUX_CENTRAL && vf != TG_FLUX_RANOCHA && vf != TG_FLUX_SHIMA_ETAL &&
        vf != TG_FLUX_CHANDRASHEKAR)
      return fail(nullptr, TG_ERR_UNSUPPORTED,
                  "curvilinear meshes: volume flux must be central, ranocha, shima_etal or "
                  "chandrashekar");
    if (sf == TG_FLUX_HLLC || sf == TG_FLUX_HLLE)
      return fail(nullptr, TG_ERR_UNSUPPORTED, "curvilinear meshes: flux_hllc / flux_hlle");
    if (cfg->nmortars != 0)
      return fail(nullptr, TG_ERR_UNSUPPORTED, "curvilinear meshes: no mortars");
    if (!cfg->contravariant_vectors)
      return fail(nullptr, TG_ERR_INVALID_ARGUMENT,
                  "curvilinear meshes need contravariant_vectors");
    const int64_t nn = D == 2 ? (int64_t)N * N : (int64_t)N * N * N;
    for (int64_t k = 0; k < cfg->nelements * nn; ++k)
      if (!(cfg->inverse_jacobian[k] > 0.0))
        return fail(nullptr, TG_ERR_UNSUPPORTED,
                    "curvilinear meshes: the mapping must preserve orientation (inverse Jacobian "
                    "> 0 at every node)");
  }
  int epb = curved ? tg::curved_epb(N)
                   : (cfg->elements_per_block > 0
                          ? cfg->elements_per_block
                          : (mixed ? default_epb_mixed(D, N) : default_epb(D, N)));
  if (!curved && (mixed ? !supported_epb_mixed(D, N, epb) : !supported_epb(D, N, epb)))
    return fail(nullptr, TG_ERR_UNSUPPORTED, "elements_per_block %d not compiled for %dD N=%d", epb,
                D, N);

  tg_ctx* c = new tg_ctx();
  c->D = D;
  c->N = N;
  c->NN = D == 2 ? N * N : N * N * N;
  c->NV = D + 2;
  c->E = cfg->nelements;
  c->ndofs = c->E * c->NN;
  c->nvalues = c->ndofs * c->NV;
  c->vi = cfg->volume_integral;
  c->fp64 = cfg->precision == TG_PRECISION_FP64;
  c->epb = epb;
  c->device = cfg->device;
  c->curved = curved;

  // ---- face-neighbour table from the interface container ----
  const int nf = 2 * D;
  std::vector<int32_t> nbr((size_t)c->E * nf, -1);
  for (int64_t f = 0; f < cfg->ninterfaces; ++f) {
    const int64_t l = cfg->neighbor_ids[2 * f] - 1, r = cfg->neighbor_ids[2 * f + 1] - 1;
    const int64_t o = cfg->orientations[f] - 1;
    if (l < 0 || l >= c->E || r < 0 || r >= c->E || o < 0 || o >= D) {
      delete c;
      return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "interface %lld out of range", (long long)f);
    }
    int32_t& a = nbr[l * nf + 2 * o + 1];
    int32_t& b = nbr[r * nf + 2 * o];
    if (a != -1 || b != -1) {
      delete c;
      return fail(nullptr, TG_ERR_UNSUPPORTED, "element face used by two interfaces");
    }
    a = (int32_t)r;
    b = (int32_t)l;
  }
  // ---- L2 mortars: mark their element faces (-2); their slots are numbered
  //      after the boundary faces below ----
  const int ns = 1 << (D - 1);
  const int64_t nm = cfg->nmortars;
  if (nm < 0 || (nm > 0 && (!cfg->mortar_neighbor_ids || !cfg->mortar_large_sides ||
                            !cfg->mortar_orientations || !cfg->mortar_forward_upper ||
                            !cfg->mortar_forward_lower || !cfg->mortar_reverse_upper ||
                            !cfg->mortar_reverse_lower))) {
    delete c;
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT,
                "mortars need neighbor_ids, large_sides, orientations and the mortar matrices");
  }
  std::vector<int32_t> mtab((size_t)nm * (ns + 3)), mnbr((size_t)nm * (ns + 1) * 4, -1);
  std::vector<int64_t> mface((size_t)nm * (ns + 1));  // element face (e * 2D + dir) of each slot
  for (int64_t m = 0; m < nm; ++m) {
    const int64_t o = cfg->mortar_orientations[m] - 1, ls = cfg->mortar_large_sides[m];
    if (o < 0 || o >= D || (ls != 1 && ls != 2)) {
      delete c;
      return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "mortar %lld: invalid orientation or large side",
                  (long long)m);
    }
    const int dir_large = ls == 1 ? (int)(2 * o + 1) : (int)(2 * o);
    int64_t ids[5];
    for (int q = 0; q <= ns; ++q) {
      ids[q] = cfg->mortar_neighbor_ids[m * (ns + 1) + q] - 1;
      if (ids[q] < 0 || ids[q] >= c->E) {
        delete c;
        return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "mortar %lld: element out of range",
                    (long long)m);
      }
      const int64_t face = ids[q] * nf + (q < ns ? (dir_large ^ 1) : dir_large);
      if (nbr[face] != -1) {
        delete c;
        return fail(nullptr, TG_ERR_UNSUPPORTED, "element face used by an interface and a mortar");
      }
      nbr[face] = -2;
      mface[m * (ns + 1) + q] = face;
      mtab[m * (ns + 3) + q] = (int32_t)ids[q];
    }
    mtab[m * (ns + 3) + ns + 1] = ls == 1 ? 0 : 1;
    mtab[m * (ns + 3) + ns + 2] = (int32_t)o;
    for (int q = 0; q < ns; ++q) {
      mnbr[(m * (ns + 1) + q) * 4] = (int32_t)ids[ns];
      mnbr[(m * (ns + 1) + ns) * 4 + q] = (int32_t)ids[q];
    }
  }
  // faces without interface or mortar are boundaries of a non-periodic mesh
  // and need a boundary condition for their direction
  bool has_dirichlet = false;
  for (int dir = 0; dir < nf; ++dir) {
    const int bc = cfg->boundary_conditions[dir];
    if (bc < TG_BOUNDARY_PERIODIC || bc > TG_BOUNDARY_SLIP_WALL) {
      delete c;
      return fail(nullptr, TG_ERR_INVALID_ARGUMENT, "boundary condition %d of direction %d", bc, dir);
    }
    has_dirichlet |= bc == TG_BOUNDARY_DIRICHLET;
  }
  if (curved)
    for (int dir = 0; dir < nf; ++dir)
      if (cfg->boundary_conditions[dir] == TG_BOUNDARY_SLIP_WALL) {
        delete c;
        return fail(nullptr, TG_ERR_UNSUPPORTED,
                    "curvilinear meshes: periodic or Dirichlet boundaries only");
      }
  for (size_t k = 0; k < nbr.size(); ++k)
    if (nbr[k] == -1 && cfg->boundary_conditions[k % nf] == TG_BOUNDARY_PERIODIC) {
      delete c;
      return fail(nullptr, TG_ERR_UNSUPPORTED,
                  "element face without interface, mortar or boundary condition (direction %d)",
                  (int)(k % nf));
    }
  if (has_dirichlet && (!cfg->node_coordinates || cfg->boundary_value_function < TG_IC_CONSTANT ||
                        cfg->boundary_value_function > TG_IC_GAUSSIAN_BLAST)) {
    delete c;
    return fail(nullptr, TG_ERR_INVALID_ARGUMENT,
                "Dirichlet boundaries need node coordinates and a valid boundary_value_function");
  }
  // boundary faces: numbered in element order, nbr = -1 - number
  std::vector<int32_t> bface;
  for (size_t k = 0; k < nbr.size(); ++k)
    if (nbr[k] == -1) {
      const int32_t b = (int32_t)(bface.size() / 2);
      bface.push_back((int32_t)(k / nf));
      bface.push_back((int32_t)(k % nf));
      nbr[k] = -1 - b;
    }
  c->nbound = (int64_t)bface.size() / 2;
  c->nmortar = nm;
  c->nmface = nm * (ns + 1);
  for (int64_t sl = 0; sl < c->nmface; ++sl) nbr[mface[sl]] = (int32_t)(-1 - (c->nbound + sl));

  // ---- node coordinates along each axis (tensor-product TreeMesh elements) ----
  std::vector<double> xline;
  if (cfg->node_coordinates && !curved) {
    xline.resize((size_t)c->E * D * N);
    const double* X = cfg->node_coordinates;
    for (int64_t e = 0; e < c->E; ++e)
      for (int q = 0; q < c->NN; ++q) {
        const int idx[3] = {q % N, (q / N) % N, q / (N * N)};
        for (int d = 0; d < D; ++d) {
          const double x = X[((size_t)e * c->NN + q) * D + d];
          double& slot = xline[((size_t)e * D + d) * N + idx[d]];
          bool first = true;
          for (int dd = 0; dd < D; ++dd)
            if (dd != d && idx[dd] != 0) first = false;
          if (first)
            slot = x;
          else if (slot != x) {
            delete c;
            return fail(nullptr, TG_ERR_UNSUPPORTED, "node coordinates are not a tensor product");
          }
        }
      }
  }

  // ---- parameters ----
  DgParams& P = c->P;
  P.nelements = c->E;
  P.gamma = cfg->gamma;
  P.inv_gamma_minus_one = 1.0 / (cfg->gamma - 1.0);
  for (int i = 0; i < N; ++i) {
    P.nodes[i] = cfg->nodes[i];
    P.inv_weights[i] = cfg->inverse_weights[i];
    c->weights.push_back(cfg->weights[i]);
  }
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b) {
      // Julia column-major (a, b) -> a + b * N
      P.Dhat[a * N + b] = cfg->derivative_hat[a + b * N];
      P.Dsplit[a * N + b] = cfg->derivative_split[a + b * N];
      P.Vinv[a * N + b] = cfg->inverse_vandermonde_legendre[a + b * N];
    }
  P.volume_flux = cfg->volume_flux;
  P.surface_flux = cfg->surface_flux;
  P.fv_flux = cfg->volume_flux_fv;
  P.source = cfg->source_terms;
  for (int dir = 0; dir < 6; ++dir) P.bc[dir] = dir < nf ? cfg->boundary_conditions[dir] : 0;
  P.bc_ic = cfg->boundary_value_function;
  for (int k = 0; k < 4; ++k) P.bc_par[k] = cfg->boundary_value_params[k];
  P.alpha_max = cfg->alpha_max;
  P.alpha_min = cfg->alpha_min;
  P.alpha_smooth = cfg->alpha_smooth;
  // indicators.jl:128-131 and calc_volume_integral.jl:242-245
  P.hg_threshold = 0.5 * std::pow(10.0, -1.8 * std::pow((double)N, 0.25));
  P.hg_parameter_s = std::log((1 - 0.0001) / 0.0001);
  P.alpha_atol = c->fp64 ? std::max(100 * 2.220446049250313e-16, std::pow(2.220446049250313e-16, 0.75))
                         : (double)std::max(100 * 1.1920929e-07f, std::pow(1.1920929e-07f, 0.75f));

  // ---- device allocations ----
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) {
    delete c;
    return fail(nullptr, TG_ERR_CUDA, "cudaSetDevice(%d): %s", cfg->device, cudaGetErrorString(e));
  }
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    free_ctx(c);
    return fail(nullptr, TG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  // stream-ordered allocations from the device's context pool (cudaMalloc if
  // the pool is unavailable or refuses for another reason than memory, e.g.
  // after a device reset); the stream is synchronised once they are made
  cudaMemPool_t pool = context_pool(c->device);
#define ALLOC(ptr, bytes)                                                                 \
  do {                                                                                    \
    e = cudaErrorNotSupported;                                                            \
    if (pool) {                                                                           \
      e = cudaMallocFromPoolAsync((void**)&(ptr), (bytes), pool, c->stream);              \
      if (e == cudaSuccess) c->pool_ptrs.push_back((void*)(ptr));                         \
      else if (e != cudaErrorMemoryAllocation) cudaGetLastError();                        \
    }                                                                                     \
    if (e != cudaSuccess && e != cudaErrorMemoryAllocation)                               \
      e = cudaMalloc((void**)&(ptr), (bytes)); /* no pool, or a pool that went away */    \
    if (e != cudaSuccess) {                                                               \
      free_ctx(c);                                                                        \
      return fail(nullptr, TG_ERR_CUDA, "device allocation (%zu bytes): %s",              \
                  (size_t)(bytes), cudaGetErrorString(e));                                \
    }                                                                                     \
  } while (0)
  const size_t vb = sizeof(double) * (size_t)c->nvalues;
  ALLOC(c->d_u[0], vb);
  ALLOC(c->d_u[1], vb);
  ALLOC(c->d_utmp, rsize(c) * (size_t)c->nvalues);
  // padded: the stage kernels' bulk copies read neighbour rows in 16-byte groups
  ALLOC(c->d_nbr, sizeof(int32_t) * nbr.size() + 16);
  if (c->nbound > 0) ALLOC(c->d_bface, sizeof(int32_t) * bface.size());
  if (!c->fp64 && c->nbound + c->nmface > 0)
    ALLOC(c->d_ghost, sizeof(float2) * (size_t)(c->nbound + c->nmface) * (c->NN / N) * c->NV);
  std::vector<double> mmat;
  if (nm > 0) {
    ALLOC(c->d_mtab, sizeof(int32_t) * mtab.size());
    ALLOC(c->d_mnbr, sizeof(int32_t) * mnbr.size());
    ALLOC(c->d_mmat, sizeof(double) * 4 * N * N);
    if (!c->fp64) ALLOC(c->d_mmat32, sizeof(float) * 4 * N * N);
    if (c->fp64) ALLOC(c->d_mflux, sizeof(double) * (size_t)c->nmface * (c->NN / N) * c->NV);
    // row-major copies of the column-major n x n mortar matrices
    const double* src[4] = {cfg->mortar_forward_lower, cfg->mortar_forward_upper,
                            cfg->mortar_reverse_lower, cfg->mortar_reverse_upper};
    mmat.resize((size_t)4 * N * N);
    for (int k = 0; k < 4; ++k)
      for (int a = 0; a < N; ++a)
        for (int b = 0; b < N; ++b) mmat[(size_t)k * N * N + a * N + b] = src[k][a + b * N];
  }
  ALLOC(c->d_invj, sizeof(double) * c->E);
  for (int64_t k = 0; k < c->E; ++k) {
    // element volume (2 / inverse_jacobian)^d: the mesh volume analysis normalises by
    double h = 2.0 / cfg->inverse_jacobian[k], v = h;
    for (int d = 1; d < D; ++d) v *= h;
    c->total_volume += v;
  }
  ALLOC(c->d_weights, sizeof(double) * N);
  ALLOC(c->d_clock, sizeof(Clock));
  ALLOC(c->d_status, sizeof(int32_t));
  ALLOC(c->d_speed, sizeof(unsigned long long));
  ALLOC(c->d_sums, sizeof(double) * 16);
  if (!xline.empty()) ALLOC(c->d_xline, sizeof(double) * xline.size());
  if (c->vi == VI_HG) {
    ALLOC(c->d_alpha_raw, rsize(c) * (c->E + kElemPad));  // padded as d_alpha_sm
    ALLOC(c->d_alpha, sizeof(double) * c->E);
    // read in whole 16-byte groups by the bulk copies of the 2D stage kernel
    if (!c->fp64) ALLOC(c->d_alpha_sm, sizeof(float) * (c->E + kElemPad));
    if (!c->fp64 && D == 2 && !curved) ALLOC(c->d_rp, sizeof(float) * c->ndofs);
  }
  std::vector<float> invj_f, xline_f;
  std::vector<float4> sc0, scn;
  std::vector<int8_t> scls;
  if (!c->fp64) {
    invj_f.resize(c->E);
    for (int64_t k = 0; k < c->E; ++k) invj_f[k] = (float)cfg->inverse_jacobian[k];
    xline_f.assign(xline.begin(), xline.end());
    ALLOC(c->d_invj_f, sizeof(float) * (c->E + kElemPad));  // padded as d_alpha_sm
    if (!xline_f.empty()) {
      ALLOC(c->d_xline_f, sizeof(float) * xline_f.size());
      if (c->P.source == SRC_CONVERGENCE_TEST) {
        // source phase pi (sum_d x_d - t) of the mixed path, split into the
        // first node of each element (FP64 -> float-float sin/cos) and the
        // node offsets from it, which are the same for all elements of one
        // size (one table per size class; checked)
        auto ffsc = [](double ph) {
          const double sn = std::sin(M_PI * ph), cs = std::cos(M_PI * ph);
          const float sh = (float)sn, ch = (float)cs;
          return make_float4(sh, ch, (float)(sn - (double)sh), (float)(cs - (double)ch));
        };
        sc0.resize(c->E);
        scls.resize(c->E);
        std::vector<double> cls_invj;   // inverse Jacobian of each size class
        std::vector<int64_t> cls_elem;  // its first element
        for (int64_t e2 = 0; e2 < c->E; ++e2) {
          size_t k = 0;
          while (k < cls_invj.size() && cls_invj[k] != cfg->inverse_jacobian[e2]) ++k;
          if (k == cls_invj.size()) {
            if (k == 64) {
              free_ctx(c);
              return fail(nullptr, TG_ERR_UNSUPPORTED,
                          "mixed precision source terms: more than 64 element sizes");
            }
            cls_invj.push_back(cfg->inverse_jacobian[e2]);
            cls_elem.push_back(e2);
          }
          scls[e2] = (int8_t)k;
          double ph = 0;
          for (int d = 0; d < D; ++d) {
            const double* xl = &xline[((size_t)e2 * D + d) * N];
            const double* x1 = &xline[((size_t)cls_elem[k] * D + d) * N];
            ph += xl[0];
            for (int i = 0; i < N; ++i)
              if (std::fabs((xl[i] - xl[0]) - (x1[i] - x1[0])) > 1e-12 * std::fabs(x1[N - 1] - x1[0])) {
                free_ctx(c);
                return fail(nullptr, TG_ERR_UNSUPPORTED,
                            "mixed precision source terms need tensor-product elements of "
                            "regular node spacing");
              }
          }
          sc0[e2] = ffsc(ph);
        }
        int NN = 1;
        for (int d = 0; d < D; ++d) NN *= N;
        scn.resize(cls_elem.size() * NN);
        for (size_t k = 0; k < cls_elem.size(); ++k)
          for (int q = 0; q < NN; ++q) {
            const double* x1 = &xline[(size_t)cls_elem[k] * D * N];
            double ph = 0;
            for (int d = 0, r = q; d < D; ++d, r /= N) ph += x1[(size_t)d * N + r % N] - x1[(size_t)d * N];
            scn[k * NN + q] = ffsc(ph);
          }
        ALLOC(c->d_sc0, sizeof(float4) * sc0.size());
        ALLOC(c->d_scn, sizeof(float4) * scn.size());
        ALLOC(c->d_scls, sizeof(int8_t) * scls.size());
      }
    }
  }
#undef ALLOC
  // the pool allocations are complete before any other stream touches them
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    free_ctx(c);
    return fail(nullptr, TG_ERR_CUDA, "context allocations: %s", cudaGetErrorString(e));
  }
  if (!c->fp64) {
    cudaMemset(c->d_invj_f, 0, sizeof(float) * (c->E + kElemPad));
    cudaMemcpy(c->d_invj_f, invj_f.data(), sizeof(float) * c->E, cudaMemcpyHostToDevice);
    if (!xline_f.empty()) {
      cudaMemcpy(c->d_xline_f, xline_f.data(), sizeof(float) * xline_f.size(),
                 cudaMemcpyHostToDevice);
      if (!sc0.empty()) {
        cudaMemcpy(c->d_sc0, sc0.data(), sizeof(float4) * sc0.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->d_scn, scn.data(), sizeof(float4) * scn.size(), cudaMemcpyHostToDevice);
        cudaMemcpy(c->d_scls, scls.data(), sizeof(int8_t) * scls.size(), cudaMemcpyHostToDevice);
      }
    }
  }
  cudaMemcpy(c->d_nbr, nbr.data(), sizeof(int32_t) * nbr.size(), cudaMemcpyHostToDevice);
  cudaMemset(c->d_nbr + nbr.size(), 0, 16);
  if (c->nbound > 0)
    cudaMemcpy(c->d_bface, bface.data(), sizeof(int32_t) * bface.size(), cudaMemcpyHostToDevice);
  if (nm > 0) {
    cudaMemcpy(c->d_mtab, mtab.data(), sizeof(int32_t) * mtab.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_mnbr, mnbr.data(), sizeof(int32_t) * mnbr.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(c->d_mmat, mmat.data(), sizeof(double) * mmat.size(), cudaMemcpyHostToDevice);
    if (!c->fp64) {
      std::vector<float> m32(mmat.begin(), mmat.end());
      cudaMemcpy(c->d_mmat32, m32.data(), sizeof(float) * m32.size(), cudaMemcpyHostToDevice);
    }
  }
  cudaMemcpy(c->d_invj, cfg->inverse_jacobian, sizeof(double) * c->E, cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_weights, c->weights.data(), sizeof(double) * N, cudaMemcpyHostToDevice);
  if (!xline.empty())
    cudaMemcpy(c->d_xline, xline.data(), sizeof(double) * xline.size(), cudaMemcpyHostToDevice);
  cudaMemset(c->d_status, 0, sizeof(int32_t));
  cudaMemset(c->d_clock, 0, sizeof(Clock));
  cudaMemset(c->d_utmp, 0, rsize(c) * (size_t)c->nvalues);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    free_ctx(c);
    return fail(nullptr, TG_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
  }
  P.nbr = c->d_nbr;
  P.inv_jac = c->d_invj;
  P.xline = c->d_xline;
  P.nbc = (int32_t)c->nbound;
  P.mflux = c->d_mflux;
  P.mnbr = c->d_mnbr;
  // single-precision copy of the parameters for the mixed path
  MixedParams& M = c->MP;
  M.nelements = P.nelements;
  M.gamma = (float)P.gamma;
  M.inv_gamma_minus_one = (float)P.inv_gamma_minus_one;
  M.eos.gamma = (float)P.gamma;
  M.eos.gm1 = (float)(P.gamma - 1.0);
  M.eos.gm1_lo = (float)((P.gamma - 1.0) - (double)M.eos.gm1);
  M.eos.igm1 = (float)P.inv_gamma_minus_one;
  M.eos.gigm1 = (float)(P.gamma * P.inv_gamma_minus_one);
  for (int k = 0; k < MAXN; ++k) M.inv_weights[k] = (float)P.inv_weights[k];
  for (int k = 0; k < MAXN * MAXN; ++k) {
    M.Dhat[k] = (float)P.Dhat[k];
    M.Dsplit[k] = (float)P.Dsplit[k];
    M.Vinv[k] = (float)P.Vinv[k];
  }
  M.volume_flux = P.volume_flux;
  M.surface_flux = P.surface_flux;
  M.fv_flux = P.fv_flux;
  M.source = P.source;
  M.alpha_max = (float)P.alpha_max;
  M.alpha_min = (float)P.alpha_min;
  M.alpha_atol = (float)P.alpha_atol;
  M.hg_threshold = (float)P.hg_threshold;
  M.hg_parameter_s = (float)P.hg_parameter_s;
  M.alpha_smooth = P.alpha_smooth;
  M.nbr = c->d_nbr;
  M.inv_jac = c->d_invj_f;
  M.xline = c->d_xline_f;
  M.sc0 = c->d_sc0;
  M.scn = c->d_scn;
  M.scls = c->d_scls;
  M.has_direct = c->nmortar > 0;
  for (int dir = 0; dir < 6; ++dir) {
    M.bc[dir] = P.bc[dir];
    M.has_direct |= P.bc[dir] == BC_SLIP_WALL;
  }
  M.nbc = (int32_t)c->nbound;
  M.ghost = c->d_ghost;
  M.mnbr = c->d_mnbr;
  // 3D polydeg 3 without shock capturing: the persistent kernel with 2
  // elements per block is the default (at 32^3 on the MMS mesh 0.169 ms per
  // stage against the per-block kernel's 0.188 with 4 elements; both give the
  // same bits)
  if (!c->fp64 && !curved && c->D == 3 && c->N == 4 && cfg->elements_per_block <= 0 &&
      c->vi != VI_HG)
    c->epb = 2;
  if (curved) {
    int rc = curved_setup(c, cfg);
    if (rc != TG_OK) {
      free_ctx(c);
      return rc;
    }
  }
  *out = c;
  return TG_OK;
}

int tg_ctx_destroy(tg_ctx* ctx) {
  if (!ctx) return TG_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  free_ctx(ctx);
  return TG_OK;
}

int tg_ndofs(const tg_ctx* ctx, int64_t* ndofs, int64_t* nvalues) {
  if (!ctx) return TG_ERR_INVALID_ARGUMENT;
  if (ndofs) *ndofs = ctx->ndofs;
  if (nvalues) *nvalues = ctx->nvalues;
  return TG_OK;
}

// Autotuner: times one stage for every elements-per-block value the element
// kernel is built with for this (D, N) and keeps the fastest.  The timed
// launches read the current state and write only what is dead between steps
// (the other state buffer and the 2N register), with a scratch clock (dt = 0)
// and status word and no wave-speed reduction, so the solution is unchanged.
int tg_ctx_autotune(tg_ctx* c, int32_t iters, int32_t* best_epb, double* ms_per_stage) {
  if (c && c->curved)
    return fail(c, TG_ERR_UNSUPPORTED, "not available for curvilinear meshes");
  if (!c || iters <= 0) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  const bool mixed = !c->fp64;
  std::vector<int> cand;
  for (int e : {mixed ? default_epb_mixed(c->D, c->N) : default_epb(c->D, c->N), 2, 4, 8, 16, 32})
    if (std::find(cand.begin(), cand.end(), e) == cand.end() &&
        (mixed ? supported_epb_mixed(c->D, c->N, e) : supported_epb(c->D, c->N, e)))
      cand.push_back(e);
  Clock* d_clk = nullptr;
  int32_t* d_st = nullptr;
  CUDA_TRY(c, cudaMalloc((void**)&d_clk, sizeof(Clock)));
  if (cudaMalloc((void**)&d_st, sizeof(int32_t)) != cudaSuccess) {
    cudaFree(d_clk);
    return fail(c, TG_ERR_CUDA, "autotune: allocation failed");
  }
  cudaMemsetAsync(d_clk, 0, sizeof(Clock), c->stream);
  cudaMemsetAsync(d_st, 0, sizeof(int32_t), c->stream);
  Clock* keep_clock = c->d_clock;
  int32_t* keep_status = c->d_status;
  const int keep_epb = c->epb;
  int rc = indicator(c, c->d_u[c->cur]);  // blending factors of the current state (HG)
  c->d_clock = d_clk;
  c->d_status = d_st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = keep_epb;
  float best_ms = 0;
  for (size_t k = 0; k < cand.size() && rc == TG_OK; ++k) {
    c->epb = cand[k];
    for (int w = 0; w < 2 && rc == TG_OK; ++w)
      rc = launch_kernel(c, MODE_STAGE, c->d_u[c->cur], c->d_u[c->cur ^ 1], nullptr, 0.0, 1, false);
    cudaEventRecord(e0, c->stream);
    for (int it = 0; it < iters && rc == TG_OK; ++it)
      rc = launch_kernel(c, MODE_STAGE, c->d_u[c->cur], c->d_u[c->cur ^ 1], nullptr, 0.0, 1, false);
    cudaEventRecord(e1, c->stream);
    if (rc != TG_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = fail(c, TG_ERR_CUDA, "autotune: stage launch failed");
      break;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= iters;
    if (k == 0 || ms < best_ms) {
      best = cand[k];
      best_ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(c->stream);
  c->d_clock = keep_clock;
  c->d_status = keep_status;
  cudaFree(d_clk);
  cudaFree(d_st);
  c->epb = rc == TG_OK ? best : keep_epb;
  for (int p = 0; p < 2; ++p)
    if (c->graph[p]) {
      cudaGraphExecDestroy(c->graph[p]);
      c->graph[p] = nullptr;
    }
  if (rc) return rc;
  if (best_epb) *best_epb = best;
  if (ms_per_stage) *ms_per_stage = best_ms;
  return TG_OK;
}

int tg_elements_per_block(const tg_ctx* ctx, int32_t* epb) {
  if (!ctx || !epb) return TG_ERR_INVALID_ARGUMENT;
  *epb = ctx->epb;
  return TG_OK;
}

// Device address of page-locked host memory (cudaHostAlloc / cudaHostRegister),
// or null for pageable memory.  The mixed path's conversion kernels read and
// write such buffers directly (over NVLink-C2C on GB300) instead of staging
// them through a device copy first.
static const void* pinned_device_ptr(const void* host) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();  // pageable memory unknown to CUDA: not an error here
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int tg_upload_state(tg_ctx* c, const double* u_host) {
  if (!c || !u_host) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t vb = sizeof(double) * c->nvalues;
  const void* pinned = c->fp64 ? nullptr : pinned_device_ptr(u_host);
  if (c->fp64) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_u[c->cur], u_host, vb, cudaMemcpyHostToDevice, c->stream));
  } else if (pinned) {
    int rc = import_state(c, (const double*)pinned, c->d_u[c->cur]);
    if (rc) return rc;
  } else {
    int rc = ensure(c, (void**)&c->d_stage64, vb);
    if (rc) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->d_stage64, u_host, vb, cudaMemcpyHostToDevice, c->stream));
    rc = import_state(c, c->d_stage64, c->d_u[c->cur]);
    if (rc) return rc;
  }
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  c->uploaded = true;
  c->clock_valid = false;
  if (c->fp64) c->rp_valid = false;
  return TG_OK;
}

int tg_download_state(tg_ctx* c, double* u_host) {
  if (!c || !u_host) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  if (!c->fp64) {
    if (void* pinned = const_cast<void*>(pinned_device_ptr(u_host))) {
      launch_from_ff(c, c->d_u[c->cur], (double*)pinned);
      CUDA_TRY(c, cudaGetLastError());
      CUDA_TRY(c, cudaStreamSynchronize(c->stream));
      return TG_OK;
    }
  }
  int rc;
  const double* src = export_state(c, &rc);
  if (rc) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(u_host, src, sizeof(double) * c->nvalues, cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

// ---- host transfers overlapping the stepping ---------------------------------
static int xfer_setup(tg_ctx* c, int32_t slot, bool out) {
  if (slot < 0 || slot > 1) return fail(c, TG_ERR_INVALID_ARGUMENT, "transfer slot must be 0 or 1");
  CUDA_TRY(c, cudaSetDevice(c->device));
  for (int k = 0; k < 2; ++k)
    if (!c->xstream[k]) CUDA_TRY(c, cudaStreamCreateWithFlags(&c->xstream[k], cudaStreamNonBlocking));
  for (cudaEvent_t* ev : {&c->ev_in_copied[slot], &c->ev_in_used[slot], &c->ev_out_ready[slot],
                          &c->ev_out_done[slot]})
    if (!*ev) CUDA_TRY(c, cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  double** buf = out ? &c->d_xout[slot] : &c->d_xin[slot];
  if (!*buf) CUDA_TRY(c, cudaMalloc((void**)buf, sizeof(double) * c->nvalues));
  return TG_OK;
}

int tg_prefetch_state(tg_ctx* c, int32_t slot, const double* u_host) {
  if (!c || !u_host) return TG_ERR_INVALID_ARGUMENT;
  int rc = xfer_setup(c, slot, false);
  if (rc) return rc;
  // the slot's previous contents must have been loaded before they are replaced
  if (c->in_used_rec[slot]) CUDA_TRY(c, cudaStreamWaitEvent(c->xstream[0], c->ev_in_used[slot], 0));
  CUDA_TRY(c, cudaMemcpyAsync(c->d_xin[slot], u_host, sizeof(double) * c->nvalues,
                              cudaMemcpyHostToDevice, c->xstream[0]));
  CUDA_TRY(c, cudaEventRecord(c->ev_in_copied[slot], c->xstream[0]));
  c->in_pending[slot] = true;
  return TG_OK;
}

int tg_load_prefetched(tg_ctx* c, int32_t slot) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  if (slot < 0 || slot > 1 || !c->in_pending[slot])
    return fail(c, TG_ERR_STATE, "no state prefetched into slot %d", slot);
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_in_copied[slot], 0));
  int rc = import_state(c, c->d_xin[slot], c->d_u[c->cur]);
  if (rc) return rc;
  CUDA_TRY(c, cudaEventRecord(c->ev_in_used[slot], c->stream));
  c->in_used_rec[slot] = true;
  c->in_pending[slot] = false;
  c->uploaded = true;
  c->clock_valid = false;  // (import_state keeps the indicator input valid)
  return TG_OK;
}

int tg_fetch_state(tg_ctx* c, int32_t slot, double* u_host) {
  if (!c || !u_host) return TG_ERR_INVALID_ARGUMENT;
  int rc = xfer_setup(c, slot, true);
  if (rc) return rc;
  // the slot's previous copy to the host must have finished before it is reused
  if (c->out_done_rec[slot]) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_out_done[slot], 0));
  if (c->fp64) {
    CUDA_TRY(c, cudaMemcpyAsync(c->d_xout[slot], c->d_u[c->cur], sizeof(double) * c->nvalues,
                                cudaMemcpyDeviceToDevice, c->stream));
  } else {
    launch_from_ff(c, c->d_u[c->cur], c->d_xout[slot]);
    CUDA_TRY(c, cudaGetLastError());
  }
  CUDA_TRY(c, cudaEventRecord(c->ev_out_ready[slot], c->stream));
  CUDA_TRY(c, cudaStreamWaitEvent(c->xstream[1], c->ev_out_ready[slot], 0));
  CUDA_TRY(c, cudaMemcpyAsync(u_host, c->d_xout[slot], sizeof(double) * c->nvalues,
                              cudaMemcpyDeviceToHost, c->xstream[1]));
  CUDA_TRY(c, cudaEventRecord(c->ev_out_done[slot], c->xstream[1]));
  c->out_done_rec[slot] = true;
  return TG_OK;
}

int tg_transfer_wait(tg_ctx* c, int32_t slot, int32_t direction) {
  if (!c || slot < 0 || slot > 1 || direction < 0 || direction > 1) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const cudaEvent_t ev = direction == 0 ? c->ev_in_copied[slot] : c->ev_out_done[slot];
  const bool rec = direction == 0 ? (c->in_pending[slot] || c->in_used_rec[slot]) : c->out_done_rec[slot];
  if (ev && rec) CUDA_TRY(c, cudaEventSynchronize(ev));
  return TG_OK;
}

int tg_transfer_join(tg_ctx* c) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  for (int k = 0; k < 2; ++k) {
    if (c->out_done_rec[k]) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_out_done[k], 0));
    if (c->in_pending[k]) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, c->ev_in_copied[k], 0));
  }
  return TG_OK;
}

int tg_state_device_ptr(tg_ctx* c, double** u_dev) {
  if (!c || !u_dev) return TG_ERR_INVALID_ARGUMENT;
  *u_dev = (double*)c->d_u[c->cur];
  c->rp_valid = false;  // the caller may write the state
  c->speed_fresh = false;
  return TG_OK;
}

int tg_rhs(tg_ctx* c, double* du_dev, const double* u_dev, double t) {
  if (!c || !du_dev || !u_dev) return TG_ERR_INVALID_ARGUMENT;
  if ((const double*)du_dev == u_dev) return fail(c, TG_ERR_INVALID_ARGUMENT, "du aliases u");
  CUDA_TRY(c, cudaSetDevice(c->device));
  const void* u_in = u_dev;
  if (!c->fp64) {
    int rc = ensure(c, (void**)&c->d_uff, sizeof(float2) * c->nvalues);
    if (rc) return rc;
    rc = import_state(c, u_dev, c->d_uff);
    if (rc) return rc;
    u_in = c->d_uff;
  }
  int rc = indicator(c, u_in);
  if (rc) return rc;
  return launch_kernel(c, MODE_RHS, u_in, nullptr, du_dev, t, 0, false);
}

int tg_rhs_host(tg_ctx* c, double* du_host, const double* u_host, double t) {
  if (!c || !du_host || !u_host) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t vb = sizeof(double) * c->nvalues;
  int rc = ensure(c, (void**)&c->d_uscratch, vb);
  if (rc) return rc;
  rc = ensure(c, (void**)&c->d_du, vb);
  if (rc) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(c->d_uscratch, u_host, vb, cudaMemcpyHostToDevice, c->stream));
  rc = tg_rhs(c, c->d_du, c->d_uscratch, t);
  if (rc) return rc;
  CUDA_TRY(c, cudaMemcpyAsync(du_host, c->d_du, vb, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_max_dt(tg_ctx* c, const double* u_dev, double* dt) {
  if (!c || !dt) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  // a caller's FP64 state, or the context state as it is stored
  int rc = reduce_speed(c, u_dev ? (const void*)u_dev : c->d_u[c->cur], !u_dev && !c->fp64,
                        c->d_speed);
  if (rc) return rc;
  unsigned long long bits = 0;
  CUDA_TRY(c, cudaMemcpyAsync(&bits, c->d_speed, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  double speed;
  std::memcpy(&speed, &bits, sizeof(speed));
  *dt = 2.0 / (c->N * speed);
  return TG_OK;
}

int tg_rk_stage(tg_ctx* c, int32_t stage, double t, double dt) {
  if (!c || stage < 0 || stage > 4) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  // the stage clock is written in stream order, without a host round trip
  clock_set_kernel<<<1, 1, 0, c->stream>>>(c->d_clock, t, dt);
  CUDA_TRY(c, cudaGetLastError());
  c->clock_valid = false;
  return enqueue_stage(c, stage, false);
}

int tg_rk_stage_part(tg_ctx* c, int32_t stage, double t, double dt, int32_t parts) {
  if (!c || stage < 0 || stage > 4 || parts < 1 || parts > 3) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  if (parts & 1) {
    clock_set_kernel<<<1, 1, 0, c->stream>>>(c->d_clock, t, dt);
    CUDA_TRY(c, cudaGetLastError());
    c->clock_valid = false;
    int rc = indicator(c, c->d_u[c->cur]);
    if (rc) return rc;
  }
  if (parts & 2) {
    int rc = launch_kernel(c, MODE_STAGE, c->d_u[c->cur], c->d_u[c->cur ^ 1], nullptr, 0.0, stage,
                           false, true);
    if (rc) return rc;
    c->cur ^= 1;
    c->rp_valid = c->d_rp != nullptr;
  }
  return TG_OK;
}

int tg_vector_create(tg_ctx* c, int64_t n, double** dev) {
  if (!c || !dev || n < 0) return TG_ERR_INVALID_ARGUMENT;
  *dev = nullptr;
  CUDA_TRY(c, cudaSetDevice(c->device));
  double* p = nullptr;
  CUDA_TRY(c, cudaMalloc(&p, sizeof(double) * (size_t)std::max<int64_t>(n, 1)));
  CUDA_TRY(c, cudaMemsetAsync(p, 0, sizeof(double) * (size_t)n, c->stream));
  c->vectors.push_back(p);
  *dev = p;
  return TG_OK;
}

int tg_vector_destroy(tg_ctx* c, double* dev) {
  if (!c || !dev) return TG_ERR_INVALID_ARGUMENT;
  auto it = std::find(c->vectors.begin(), c->vectors.end(), dev);
  if (it == c->vectors.end())
    return fail(c, TG_ERR_INVALID_ARGUMENT, "not a vector of this context");
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));  // no launch still uses it
  c->vectors.erase(it);
  CUDA_TRY(c, cudaFree(dev));
  return TG_OK;
}

int tg_vector_copy(tg_ctx* c, void* dst, const void* src, int64_t n, int32_t kind) {
  if (!c || !dst || !src || n < 0 || kind < 0 || kind > 2) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice
                           : kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  CUDA_TRY(c, cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n, k, c->stream));
  if (kind != 2) CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_lincomb(tg_ctx* c, int64_t n, double* out, double a, const double* x, double b,
               const double* y) {
  if (!c || !out || !x || n < 0) return TG_ERR_INVALID_ARGUMENT;
  if (n == 0) return TG_OK;
  CUDA_TRY(c, cudaSetDevice(c->device));
  lincomb_kernel<<<conv_blocks(n), 256, 0, c->stream>>>(n, out, a, x, b, y);
  CUDA_TRY(c, cudaGetLastError());
  return TG_OK;
}

int tg_stream(tg_ctx* c, void** stream) {
  if (!c || !stream) return TG_ERR_INVALID_ARGUMENT;
  *stream = (void*)c->stream;
  return TG_OK;
}

int tg_set_time(tg_ctx* c, double t) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  c->clock_valid = false;
  (void)t;
  return TG_OK;
}

extern "C++" {
namespace tg {
int ctx_clock_prepare(tg_ctx* c, double t0, double t_end, double cfl, bool sync) {
  if (!c->clock_valid) {
    // initialize!(StepsizeCallback): dt = cfl * max_dt(u0)
    if (!c->speed_fresh) {
      int rc = reduce_speed(c, c->d_u[c->cur], !c->fp64, &c->d_clock->speed_bits);
      if (rc) return rc;
    }
    c->speed_fresh = false;
    clock_init_kernel<<<1, 1, 0, c->stream>>>(c->d_clock, t0, t_end, cfl, c->N);
    CUDA_TRY(c, cudaGetLastError());
    c->clock_valid = true;
    c->host_steps = 0;
    c->host_steps_valid = true;
  } else {
    clock_config_kernel<<<1, 1, 0, c->stream>>>(c->d_clock, t_end, cfl);
    CUDA_TRY(c, cudaGetLastError());
  }
  if (sync) CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int ctx_view(tg_ctx* c, CtxView* v) {
  if (!c || !v) return TG_ERR_INVALID_ARGUMENT;
  v->mp = &c->MP;
  v->u[0] = c->d_u[0];
  v->u[1] = c->d_u[1];
  v->cur = c->cur;
  v->utmp = c->d_utmp;
  v->clock = c->d_clock;
  v->status = c->d_status;
  v->D = c->D;
  v->N = c->N;
  v->vi = c->vi;
  v->fp64 = c->fp64 ? 1 : 0;
  v->epb = c->epb;
  v->E = c->E;
  v->stream = c->stream;
  v->uploaded = c->uploaded;
  return TG_OK;
}

void ctx_set_cur(tg_ctx* c, int cur) {
  c->cur = cur & 1;
  c->rp_valid = false;
  c->speed_fresh = false;
  c->host_steps_valid = false;  // stepped by the ensemble
}
}  // namespace tg
}  // extern "C++"

// The clock as the host sees it after everything enqueued so far: a kernel
// writes it to mapped host memory (no copy engine), then the stream is
// synchronised.
__global__ void clock_publish_kernel(const Clock* __restrict__ src, Clock* __restrict__ dst) {
  const int* s = reinterpret_cast<const int*>(src);
  volatile int* d = reinterpret_cast<volatile int*>(dst);
  for (int k = threadIdx.x; k < (int)(sizeof(Clock) / sizeof(int)); k += blockDim.x) d[k] = s[k];
  __threadfence_system();
}

static int read_clock(tg_ctx* c, Clock* h) {
  if (!c->h_clock) {
    CUDA_TRY(c, cudaHostAlloc((void**)&c->h_clock, sizeof(Clock), cudaHostAllocMapped));
    CUDA_TRY(c, cudaHostGetDevicePointer((void**)&c->h_clock_dev, c->h_clock, 0));
  }
  clock_publish_kernel<<<1, 32, 0, c->stream>>>(c->d_clock, c->h_clock_dev);
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  std::memcpy(h, (const void*)c->h_clock, sizeof(Clock));
  return TG_OK;
}

static int capture_step_graph(tg_ctx* c, int parity) {
  const int saved = c->cur;
  const bool saved_rp = c->rp_valid, saved_speed = c->speed_fresh;
  c->cur = parity;
  // stage 0 reads rho*p of the step's input state: tg_step refreshes it
  // before launching the graphs whenever the state was set from outside
  c->rp_valid = c->d_rp != nullptr;
  cudaGraph_t g = nullptr;
  CUDA_TRY(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  clock_begin_kernel<<<1, 32, 0, c->stream>>>(c->d_clock);
  int rc = TG_OK;
  for (int s = 0; s < 5 && rc == TG_OK; ++s) rc = enqueue_stage(c, s, s == 4);
  if (rc == TG_OK) clock_end_kernel<<<1, 1, 0, c->stream>>>(c->d_clock, c->N);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->cur = saved;
  c->rp_valid = saved_rp;
  c->speed_fresh = saved_speed;  // (capture only records the launches)
  if (rc != TG_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(c, TG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&c->graph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(c, TG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return TG_OK;
}

int tg_step(tg_ctx* c, int64_t max_steps, double cfl, double t_end, double* t_inout,
            int64_t* steps_taken) {
  if (!c || !t_inout || max_steps < 0 || !(cfl > 0)) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  for (int p = 0; p < 2; ++p)
    if (!c->graph[p]) {
      int rc = capture_step_graph(c, p);
      if (rc) return rc;
    }
  int rc = tg::ctx_clock_prepare(c, *t_inout, t_end, cfl, false);  // the clock read below orders it
  if (rc) return rc;
  rc = refresh_rho_p(c);
  if (rc) return rc;
  Clock h{};
  // the step count before this call: known on the host unless something else
  // stepped the context (then read, which waits for the stream)
  if (!c->host_steps_valid) {
    rc = read_clock(c, &h);
    if (rc) return rc;
    c->host_steps = h.steps;
    c->host_steps_valid = true;
  }
  const int64_t steps0 = c->host_steps;
  int64_t launched = 0;
  const int64_t poll = 64;
  while (launched < max_steps) {
    const int64_t chunk = std::min(poll, max_steps - launched);
    for (int64_t k = 0; k < chunk; ++k) {
      CUDA_TRY(c, cudaGraphLaunch(c->graph[c->cur], c->stream));
      c->cur ^= 1;
      c->rp_valid = c->d_rp != nullptr;
    }
    launched += chunk;
    if (std::isfinite(t_end) || launched >= max_steps) {
      rc = read_clock(c, &h);
      if (rc) return rc;
      if (h.finished) break;
    }
  }
  if (launched == 0) {  // max_steps == 0: the clock as prepared
    rc = read_clock(c, &h);
    if (rc) return rc;
  }
  *t_inout = h.t;
  c->host_steps = h.steps;
  if (steps_taken) *steps_taken = h.steps - steps0;
  if (h.nan_dt) return fail(c, TG_ERR_NUMERICAL, "time step size `dt` is NaN");
  return TG_OK;
}

int tg_step_enqueue(tg_ctx* c, int64_t nsteps, double cfl, double t_end, double t_start) {
  if (!c || nsteps < 0 || !(cfl > 0)) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  for (int p = 0; p < 2; ++p)
    if (!c->graph[p]) {
      int rc = capture_step_graph(c, p);
      if (rc) return rc;
    }
  int rc = tg::ctx_clock_prepare(c, t_start, t_end, cfl, false);
  if (rc) return rc;
  rc = refresh_rho_p(c);
  if (rc) return rc;
  for (int64_t k = 0; k < nsteps; ++k) {
    CUDA_TRY(c, cudaGraphLaunch(c->graph[c->cur], c->stream));
    c->cur ^= 1;
    c->rp_valid = c->d_rp != nullptr;
  }
  c->host_steps_valid = false;  // known again at the next clock read
  return TG_OK;
}

int tg_clock_read(tg_ctx* c, double* t, int64_t* steps, int32_t* finished) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  Clock h{};
  int rc = read_clock(c, &h);
  if (rc) return rc;
  c->host_steps = h.steps;
  c->host_steps_valid = c->clock_valid;
  if (t) *t = h.t;
  if (steps) *steps = h.steps;
  if (finished) *finished = h.finished;
  if (h.nan_dt) return fail(c, TG_ERR_NUMERICAL, "time step size `dt` is NaN");
  return TG_OK;
}

int tg_integrals(tg_ctx* c, double* out) {
  if (!c || !out) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const int K = c->NV + 2;
  if (!c->d_partial) CUDA_TRY(c, cudaMalloc((void**)&c->d_partial, sizeof(double) * K * c->E));
  const int64_t nb = (c->E + 127) / 128;
  if (c->curved) {
    const int rc = c->D == 3 ? tg::launch_curved3_integrals(c->CP, c->d_u[c->cur], !c->fp64,
                                                            c->d_weights, c->d_partial, c->stream)
                             : tg::launch_curved_integrals(c->CP, c->d_u[c->cur], !c->fp64,
                                                           c->d_weights, c->d_partial, c->stream);
    if (rc != 0) return fail(c, TG_ERR_CUDA, "curvilinear integrals launch failed");
  } else if (c->fp64) {
    const double* u = (const double*)c->d_u[c->cur];
    if (c->D == 2)
      element_integrals_kernel<2, double><<<(unsigned)nb, 128, 0, c->stream>>>(
          u, c->d_invj, c->d_weights, c->E, c->N, c->P.gamma, c->d_partial);
    else
      element_integrals_kernel<3, double><<<(unsigned)nb, 128, 0, c->stream>>>(
          u, c->d_invj, c->d_weights, c->E, c->N, c->P.gamma, c->d_partial);
  } else {
    const float2* u = (const float2*)c->d_u[c->cur];
    if (c->D == 2)
      element_integrals_kernel<2, float2><<<(unsigned)nb, 128, 0, c->stream>>>(
          u, c->d_invj, c->d_weights, c->E, c->N, c->P.gamma, c->d_partial);
    else
      element_integrals_kernel<3, float2><<<(unsigned)nb, 128, 0, c->stream>>>(
          u, c->d_invj, c->d_weights, c->E, c->N, c->P.gamma, c->d_partial);
  }
  sum_rows_kernel<<<1, 256, 256 * sizeof(double), c->stream>>>(c->d_partial, c->E, K, c->d_sums);
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(out, c->d_sums, sizeof(double) * K, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_error_norms(tg_ctx* c, const double* u_dev, double t, int32_t ic, const double* params,
                   int32_t nanalyzer, const double* analyzer_vandermonde,
                   const double* analyzer_weights, double* l2, double* linf) {
  if (!c || !analyzer_vandermonde || !analyzer_weights || !l2 || !linf)
    return TG_ERR_INVALID_ARGUMENT;
  if (ic < TG_IC_CONSTANT || ic > TG_IC_GAUSSIAN_BLAST)
    return fail(c, TG_ERR_UNSUPPORTED, "error norms: the exact solution must be a device initial condition");
  if (c->curved) return fail(c, TG_ERR_UNSUPPORTED, "error norms: TreeMesh contexts only");
  if (!c->d_xline) return fail(c, TG_ERR_STATE, "error norms need the node coordinates in the config");
  if (nanalyzer < 2 || nanalyzer > 2 * MAXN - 1)
    return fail(c, TG_ERR_INVALID_ARGUMENT, "error norms: analyzer size out of range");
  if (!u_dev && !c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  CUDA_TRY(c, cudaSetDevice(c->device));
  ErrorNormArgs A{};
  A.N = c->N;
  A.NA = nanalyzer;
  A.ic = ic;
  for (int k = 0; k < 4; ++k) A.par[k] = params ? params[k] : 0.0;
  A.t = t;
  A.gamma = c->P.gamma;
  for (int a = 0; a < nanalyzer; ++a) {
    A.aw[a] = analyzer_weights[a];
    for (int k = 0; k < c->N; ++k)  // column-major [nanalyzer, n] as Trixi's analyzer.vandermonde
      A.avand[a * c->N + k] = analyzer_vandermonde[a + (size_t)k * nanalyzer];
  }
  const int NV = c->D + 2, NC = NV + c->D;
  int nna = nanalyzer;
  for (int d = 1; d < c->D; ++d) nna *= nanalyzer;
  const size_t smem = sizeof(double) * ((size_t)2 * nna * NC + 128 * 2 * NV);
  if (smem > 200 * 1024)
    return fail(c, TG_ERR_UNSUPPORTED, "error norms: analyzer too large for shared memory");
  int rc = ensure(c, (void**)&c->d_enorm, sizeof(double) * (size_t)c->E * 2 * NV);
  if (rc) return rc;
  const void* u = u_dev ? (const void*)u_dev : c->d_u[c->cur];
  const bool ff = !u_dev && !c->fp64;
#define ERRN(DD, TS)                                                                       \
  {                                                                                        \
    auto k = error_norms_kernel<DD, TS>;                                                    \
    CUDA_TRY(c, cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
    k<<<(unsigned)c->E, 128, smem, c->stream>>>((const TS*)u, c->d_xline, c->d_invj, A,      \
                                                c->d_enorm);                                \
  }
  if (c->D == 2) {
    if (ff) ERRN(2, float2) else ERRN(2, double)
  } else {
    if (ff) ERRN(3, float2) else ERRN(3, double)
  }
#undef ERRN
  sum_max_rows_kernel<<<1, 256, 256 * sizeof(double), c->stream>>>(c->d_enorm, c->E, NV,
                                                                    c->d_sums);
  CUDA_TRY(c, cudaGetLastError());
  double h[10];
  CUDA_TRY(c, cudaMemcpyAsync(h, c->d_sums, sizeof(double) * 2 * NV, cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  for (int v = 0; v < NV; ++v) {
    l2[v] = std::sqrt(h[v] / c->total_volume);
    linf[v] = h[NV + v];
  }
  return TG_OK;
}

int tg_entropy_timederivative(tg_ctx* c, double t, double* out) {
  if (c && c->curved)
    return fail(c, TG_ERR_UNSUPPORTED, "not available for curvilinear meshes");
  if (!c || !out) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  const size_t vb = sizeof(double) * c->nvalues;
  int rc = ensure(c, (void**)&c->d_du, vb);
  if (rc) return rc;
  const double* u64 = export_state(c, &rc);
  if (rc) return rc;
  rc = tg_rhs(c, c->d_du, u64, t);
  if (rc) return rc;
  const int K = c->NV + 2;  // the integrals' partial buffer has room for 2 per element
  if (!c->d_partial) CUDA_TRY(c, cudaMalloc((void**)&c->d_partial, sizeof(double) * K * c->E));
  const int64_t nb = (c->E + 127) / 128;
  if (c->D == 2)
    element_entropy_kernel<2><<<(unsigned)nb, 128, 0, c->stream>>>(u64, c->d_du, c->d_invj, c->d_weights,
                                                                   c->E, c->N, c->P.gamma, c->d_partial);
  else
    element_entropy_kernel<3><<<(unsigned)nb, 128, 0, c->stream>>>(u64, c->d_du, c->d_invj, c->d_weights,
                                                                   c->E, c->N, c->P.gamma, c->d_partial);
  sum_rows_kernel<<<1, 256, 256 * sizeof(double), c->stream>>>(c->d_partial, c->E, 2, c->d_sums);
  CUDA_TRY(c, cudaGetLastError());
  double h[2];
  CUDA_TRY(c, cudaMemcpyAsync(h, c->d_sums, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  *out = h[0] / h[1];
  return TG_OK;
}

int tg_amr_indicator(tg_ctx* c, double alpha_max, double alpha_min, int32_t alpha_smooth,
                     int32_t variable, double* alpha_host) {
  if (c && c->curved)
    return fail(c, TG_ERR_UNSUPPORTED, "not available for curvilinear meshes");
  if (!c || !alpha_host) return TG_ERR_INVALID_ARGUMENT;
  if (variable != TG_INDICATOR_DENSITY_PRESSURE && variable != TG_INDICATOR_DENSITY)
    return fail(c, TG_ERR_INVALID_ARGUMENT, "unknown indicator variable %d", variable);
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  if (!(alpha_max >= 0 && alpha_min >= 0)) return fail(c, TG_ERR_INVALID_ARGUMENT, "alpha bounds");
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure(c, (void**)&c->d_amr_raw, sizeof(double) * c->E);
  if (!rc) rc = ensure(c, (void**)&c->d_amr_alpha, sizeof(double) * c->E);
  if (rc) return rc;
  const double* u = export_state(c, &rc);
  if (!u) return rc;
  DgParams P = c->P;
  P.alpha_max = alpha_max;
  P.alpha_min = alpha_min;
  P.hg_variable = variable;
  rc = launch_indicator(c->D, c->N, true, P, u, c->d_amr_raw, c->stream);
  if (rc != 0) return fail(c, TG_ERR_CUDA, "indicator kernel launch failed (%d)", rc);
  smooth_alpha_kernel<double><<<(unsigned)((c->E + 127) / 128), 128, 0, c->stream>>>(
      c->d_amr_raw, c->d_nbr, c->E, 2 * c->D, alpha_smooth, c->P.nbc, c->d_mnbr, c->d_amr_alpha);
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(alpha_host, c->d_amr_alpha, sizeof(double) * c->E,
                              cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_amr_indicator_max(tg_ctx* c, int32_t variable, double* out_host) {
  if (c && c->curved)
    return fail(c, TG_ERR_UNSUPPORTED, "not available for curvilinear meshes");
  if (!c || !out_host) return TG_ERR_INVALID_ARGUMENT;
  if (!c->uploaded) return fail(c, TG_ERR_STATE, "no state uploaded");
  if (variable != TG_INDICATOR_DENSITY_PRESSURE && variable != TG_INDICATOR_DENSITY)
    return fail(c, TG_ERR_INVALID_ARGUMENT, "unknown indicator variable %d", variable);
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = ensure(c, (void**)&c->d_amr_alpha, sizeof(double) * c->E);
  if (rc) return rc;
  const unsigned nb = (unsigned)((c->E * 32 + 127) / 128);
  const void* u = c->d_u[c->cur];
  if (c->fp64) {
    if (c->D == 2)
      indicator_max_kernel<2, double><<<nb, 128, 0, c->stream>>>((const double*)u, c->E, c->NN,
                                                                 variable, c->P.gamma, c->d_amr_alpha);
    else
      indicator_max_kernel<3, double><<<nb, 128, 0, c->stream>>>((const double*)u, c->E, c->NN,
                                                                 variable, c->P.gamma, c->d_amr_alpha);
  } else {
    if (c->D == 2)
      indicator_max_kernel<2, float2><<<nb, 128, 0, c->stream>>>((const float2*)u, c->E, c->NN,
                                                                 variable, c->P.gamma, c->d_amr_alpha);
    else
      indicator_max_kernel<3, float2><<<nb, 128, 0, c->stream>>>((const float2*)u, c->E, c->NN,
                                                                 variable, c->P.gamma, c->d_amr_alpha);
  }
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(out_host, c->d_amr_alpha, sizeof(double) * c->E,
                              cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_adapt_state(tg_ctx* dst, tg_ctx* src, const int64_t* source_element, const int8_t* kind,
                   const double* forward_upper, const double* forward_lower,
                   const double* reverse_upper, const double* reverse_lower) {
  if ((dst && dst->curved) || (src && src->curved))
    return fail(dst, TG_ERR_UNSUPPORTED, "not available for curvilinear meshes");
  if (!dst || !src || !source_element || !kind || !forward_upper || !forward_lower ||
      !reverse_upper || !reverse_lower)
    return TG_ERR_INVALID_ARGUMENT;
  if (dst == src || dst->device != src->device || dst->D != src->D || dst->N != src->N ||
      dst->fp64 != src->fp64)
    return fail(dst, TG_ERR_INVALID_ARGUMENT,
                "adapt_state: contexts differ in device, ndims, polydeg or precision");
  if (!src->uploaded) return fail(dst, TG_ERR_STATE, "adapt_state: the source has no state");
  const int nch = 1 << dst->D, N = dst->N;
  for (int64_t e = 0; e < dst->E; ++e) {
    const int k = kind[e];
    const int64_t last = source_element[e] + (k < 0 ? nch - 1 : 0);
    if (k < -1 || k > nch || source_element[e] < 0 || last >= src->E)
      return fail(dst, TG_ERR_INVALID_ARGUMENT, "adapt_state: element %lld maps outside the source",
                  (long long)e);
  }
  AdaptMats M{};
  const double* in[4] = {forward_lower, forward_upper, reverse_lower, reverse_upper};
  for (int q = 0; q < 4; ++q)
    for (int a = 0; a < N; ++a)
      for (int b = 0; b < N; ++b) M.m[q][a * N + b] = in[q][a + b * N];
  CUDA_TRY(dst, cudaSetDevice(dst->device));
  CUDA_TRY(dst, cudaStreamSynchronize(src->stream));  // the source state is final
  if (dst->d_amap) {
    cudaFree(dst->d_amap);
    dst->d_amap = nullptr;
  }
  if (dst->d_akind) {
    cudaFree(dst->d_akind);
    dst->d_akind = nullptr;
  }
  int rc = ensure(dst, (void**)&dst->d_amap, sizeof(int64_t) * dst->E);
  if (!rc) rc = ensure(dst, (void**)&dst->d_akind, sizeof(int8_t) * dst->E);
  if (rc) return rc;
  CUDA_TRY(dst, cudaMemcpyAsync(dst->d_amap, source_element, sizeof(int64_t) * dst->E,
                                cudaMemcpyHostToDevice, dst->stream));
  CUDA_TRY(dst, cudaMemcpyAsync(dst->d_akind, kind, sizeof(int8_t) * dst->E, cudaMemcpyHostToDevice,
                                dst->stream));
  const int64_t nt = dst->E * dst->NN;
  const unsigned nb = (unsigned)((nt + 127) / 128);
  void* out = dst->d_u[dst->cur];
  const void* uo = src->d_u[src->cur];
  if (dst->fp64) {
    if (dst->D == 2)
      adapt_state_kernel<2, double><<<nb, 128, 0, dst->stream>>>((const double*)uo, (double*)out,
                                                                 dst->d_amap, dst->d_akind, dst->E, N, M);
    else
      adapt_state_kernel<3, double><<<nb, 128, 0, dst->stream>>>((const double*)uo, (double*)out,
                                                                 dst->d_amap, dst->d_akind, dst->E, N, M);
  } else {
    if (dst->D == 2)
      adapt_state_kernel<2, float2><<<nb, 128, 0, dst->stream>>>((const float2*)uo, (float2*)out,
                                                                 dst->d_amap, dst->d_akind, dst->E, N, M);
    else
      adapt_state_kernel<3, float2><<<nb, 128, 0, dst->stream>>>((const float2*)uo, (float2*)out,
                                                                 dst->d_amap, dst->d_akind, dst->E, N, M);
  }
  CUDA_TRY(dst, cudaGetLastError());
  CUDA_TRY(dst, cudaStreamSynchronize(dst->stream));
  dst->uploaded = true;
  dst->clock_valid = false;
  dst->rp_valid = false;
  dst->speed_fresh = false;
  return TG_OK;
}

int tg_alpha(tg_ctx* c, const double* u_dev, double* alpha_host) {
  if (!c || !alpha_host) return TG_ERR_INVALID_ARGUMENT;
  if (c->vi != VI_HG) return fail(c, TG_ERR_STATE, "context has no shock-capturing indicator");
  CUDA_TRY(c, cudaSetDevice(c->device));
  const void* u_in = c->d_u[c->cur];
  if (u_dev) {
    u_in = u_dev;
    if (!c->fp64) {
      int rc = ensure(c, (void**)&c->d_uff, sizeof(float2) * c->nvalues);
      if (rc) return rc;
      rc = import_state(c, u_dev, c->d_uff);
      if (rc) return rc;
      u_in = c->d_uff;
    }
  }
  int rc = indicator(c, u_in);
  if (rc) return rc;
  const int64_t nb = (c->E + 127) / 128;
  if (c->fp64)
    smooth_alpha_kernel<double><<<(unsigned)nb, 128, 0, c->stream>>>(
        (const double*)c->d_alpha_raw, c->d_nbr, c->E, 2 * c->D, c->P.alpha_smooth, c->P.nbc,
        c->d_mnbr, c->d_alpha);
  else
    smooth_alpha_kernel<float><<<(unsigned)nb, 128, 0, c->stream>>>(
        (const float*)c->d_alpha_raw, c->d_nbr, c->E, 2 * c->D, c->P.alpha_smooth, c->P.nbc,
        c->d_mnbr, c->d_alpha);
  CUDA_TRY(c, cudaGetLastError());
  CUDA_TRY(c, cudaMemcpyAsync(alpha_host, c->d_alpha, sizeof(double) * c->E, cudaMemcpyDeviceToHost,
                              c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_status(tg_ctx* c, int32_t* flags) {
  if (!c || !flags) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaMemcpyAsync(flags, c->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(c, cudaMemsetAsync(c->d_status, 0, sizeof(int32_t), c->stream));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

int tg_synchronize(tg_ctx* c) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaStreamSynchronize(c->stream));
  return TG_OK;
}

}  // extern "C"
