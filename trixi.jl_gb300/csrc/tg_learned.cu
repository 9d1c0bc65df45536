// Learned shock indicator: a small MLP that predicts the Hennemann-Gassner
// smoothness indicator of an element from its modal coefficients.
//
// Features.  The n^d modal coefficients m of density*pressure (the same
// dimension-wise inverse-Vandermonde transform as the HG indicator,
// indicators_2d.jl:50-56 / indicators_3d.jl:54-60), normalised to unit
// energy, m / |m|.
// Target.   sqrt(E) of the HG energy indicator E = max(energy fractions of the
// highest and second-highest modes) (indicators_2d.jl:58-90): the relative
// norm of the high modes, homogeneous of degree one in the normalised
// features and so well suited to a ReLU network.  The HG logistic map
// alpha = 1 / (1 + exp(-s/T (E - T))), the clipping at alpha_min and the cap
// alpha_max (indicators_2d.jl:92-100) are applied to E = prediction^2 exactly
// as to E itself.
// Fallback/judge.  Elements whose predicted sqrt(E) lies within `band` of
// sqrt(T) (where alpha switches on) or whose nodal rho*p is not positive
// take the HG alpha, which is computed from the same modes.
//
// Network: NM -> H -> H -> 1 with ReLU (2D polydeg 3: 16 -> 64 -> 64 -> 1,
// 3D: 64 -> 128 -> 128 -> 1), weights stored in BF16 for the forward pass
// with FP32 master copies, FP32 layer inputs and accumulation.  Inference and
// deployment run the two hidden layers on the tensor cores (tcgen05 BF16
// MMAs, FP32 accumulation in tensor memory), each FP32 layer input fed as a
// BF16 pair hi + lo (two MMAs into one accumulator: a 16-bit significand; a
// single BF16 rounding would erase the first layer's small-mode signal, which
// rides on the O(1) mean mode); the output layer and everything per element
// run on the CUDA cores.  Training (Adam on the mean squared error of sqrt E)
// uses the fused forward+backward kernel below on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/trixi_gb300.h"
#include "tg_dg.cuh"
#include "tg_tcgen05.cuh"

namespace tg {
void set_thread_error(const char* msg);
// Provided by tg_api.cu: state access and basis of a context.
int ctx_state_view(tg_ctx* c, const void** state, int* is_ff, int* D, int* N, int64_t* E,
                   double* gamma, const double** vinv_rowmajor, void** stream);
int ctx_set_alpha_source(tg_ctx* c, struct tg_mlp* m);
}  // namespace tg

struct tg_mlp {
  int D = 2, N = 4, NM = 16, H = 64;
  int64_t nparams = 0;
  float* d_w = nullptr;              // FP32 master parameters
  __nv_bfloat16* d_wb = nullptr;     // BF16 copy used by the kernels
  unsigned char* d_wimg = nullptr;   // d_wb as mlp_tc_kernel's shared-memory image
  size_t wimg_bytes = 0;
  float* d_g = nullptr;              // gradients
  float* d_m = nullptr;              // Adam first moments
  float* d_v = nullptr;              // Adam second moments
  float* d_x = nullptr;              // dataset features [cap][NM]
  float* d_y = nullptr;              // dataset targets [cap]
  int64_t cap = 0, count = 0;
  float* d_loss = nullptr;           // [2]: loss sum, sample count
  float* d_gpart = nullptr;          // [blocks][nparams] gradient partials of one step
  float* d_lpart = nullptr;          // [blocks] squared-error partials of one step
  int64_t part_blocks = 0;           // capacity of the partial buffers in blocks
  int64_t adam_t = 0;
  float band = 0.01f;                // half-width of the fallback zone around sqrt(T)
  double sqrt_threshold = 0.0;       // sqrt(T) of the HG indicator
  // deployment scratch
  float* d_pred = nullptr;           // [E] predicted sqrt(E)
  float* d_hg = nullptr;             // [E] HG alpha (unsmoothed)
  int32_t* d_flag = nullptr;         // [E] fallback reason (0 none, 1 band, 2 positivity)
  int64_t ecap = 0;
  unsigned long long* d_stats = nullptr;  // [3]: elements, band fallbacks, positivity fallbacks
  int32_t* d_status = nullptr;       // tensor-core wait timeouts of tg_mlp_predict
  std::string err;
};

namespace tg {

// Offsets of the parameter blocks: W1[H][NM], b1[H], W2[H][H], b2[H], w3[H], b3.
struct MlpLayout {
  int NM, H;
  __host__ __device__ int w1() const { return 0; }
  __host__ __device__ int b1() const { return H * NM; }
  __host__ __device__ int w2() const { return H * NM + H; }
  __host__ __device__ int b2() const { return H * NM + H + H * H; }
  __host__ __device__ int w3() const { return H * NM + 2 * H + H * H; }
  __host__ __device__ int b3() const { return H * NM + 3 * H + H * H; }
  __host__ __device__ int count() const { return H * NM + 3 * H + H * H + 1; }
};

__device__ __forceinline__ float wld(const __nv_bfloat16* w, int k) { return __bfloat162float(w[k]); }


// ---------------------------------------------------------------------------
// Features of every element: normalised modes, sqrt E target, HG alpha, and
// the positivity flag.  One thread per element (dimension-wise transforms in
// registers; n <= 5).
// ---------------------------------------------------------------------------
struct FeatParams {
  int64_t E;
  double gamma;
  float Vinv[MAXN * MAXN];
  float alpha_min, alpha_max, hg_threshold, hg_parameter_s;
};

// One 16-byte read-only load kept whole even where only some lanes of it are
// used (the hi halves of a float-float pair): split into 4-byte loads it
// would touch every 32-byte sector twice.
__device__ __forceinline__ float4 ldg_v4(const void* p) {
  float4 r;
  asm("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
      : "l"(p));
  return r;
}

// rho*p at node `node` (global node index e * n^d + q) of the state, and
// whether it is positive.
template <int D, typename TS>
__device__ __forceinline__ float node_rho_p(const FeatParams& P, const TS* __restrict__ u,
                                            int64_t node) {
  constexpr int NV = D + 2;
  float uu[NV];
  if constexpr (std::is_same<TS, float2>::value && NV % 2 == 0) {
    // float-float state: two values per 16-byte load (a node's values are
    // contiguous and 16-byte aligned when NV is even)
    const float4* p4 = reinterpret_cast<const float4*>(u + (size_t)node * NV);
#pragma unroll
    for (int v = 0; v < NV; v += 2) {
      const float4 x = ldg_v4(p4 + v / 2);
      uu[v] = state_value(make_float2(x.x, x.y));
      uu[v + 1] = state_value(make_float2(x.z, x.w));
    }
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) uu[v] = (float)state_value(u[(size_t)node * NV + v]);
  }
  return Euler<D, float>::density_pressure(uu, (float)P.gamma);
}

// rho*p of node k of a 2D tile staged in shared memory (4 values per node, 32
// bytes: float-float pairs or FP64), with node_rho_p's arithmetic.
template <typename TS>
__device__ __forceinline__ float staged_rho_p(const FeatParams& P, const float4* stg, int k) {
  float uu[4];
  if constexpr (std::is_same<TS, float2>::value) {
    const float4 x0 = stg[2 * k], x1 = stg[2 * k + 1];
    uu[0] = state_value(make_float2(x0.x, x0.y));
    uu[1] = state_value(make_float2(x0.z, x0.w));
    uu[2] = state_value(make_float2(x1.x, x1.y));
    uu[3] = state_value(make_float2(x1.z, x1.w));
  } else {
    const double* d = reinterpret_cast<const double*>(stg) + 4 * k;
#pragma unroll
    for (int v = 0; v < 4; ++v) uu[v] = (float)state_value(d[v]);
  }
  return Euler<2, float>::density_pressure(uu, (float)P.gamma);
}

// Modes of rho*p (a[NN], the nodal values; overwritten) normalised to unit
// energy, the HG energy indicator max(f1, f2) and positivity of rho*p at the
// nodes.
template <int D, int N>
__device__ __forceinline__ void modes_from_rho_p(const FeatParams& P, float* a, float* modes,
                                                 float& energy, bool& positive) {
  constexpr int NN = Pow<N, D>::value;
  float b[NN];
  positive = true;
#pragma unroll
  for (int q = 0; q < NN; ++q) positive &= a[q] > 0.0f;
  // multiply_scalar_dimensionwise!: x, then y, then z
  float* in = a;
  float* out = b;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int S = d == 0 ? 1 : (d == 1 ? N : N * N);
#pragma unroll
    for (int q = 0; q < NN; ++q) {
      const int i = (q / S) % N;
      const int base = q - i * S;
      float r = 0;
#pragma unroll
      for (int k = 0; k < N; ++k) r += P.Vinv[i * N + k] * in[base + k * S];
      out[q] = r;
    }
    float* t = in;
    in = out;
    out = t;
  }
  float clip2 = 0, clip1 = 0, tot = 0;
#pragma unroll
  for (int q = 0; q < NN; ++q) {
    int mx = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) mx = max(mx, (q / (d == 0 ? 1 : (d == 1 ? N : N * N))) % N);
    const float m2 = in[q] * in[q];
    if (mx <= N - 3) clip2 += m2;
    if (mx <= N - 2) clip1 += m2;
    tot += m2;
  }
  const float f1 = tot != 0.0f ? (tot - clip1) / tot : 0.0f;
  const float f2 = clip1 != 0.0f ? (clip1 - clip2) / clip1 : 0.0f;
  energy = fmaxf(f1, f2);
  const float inv = tot > 0.0f ? rsqrtf(tot) : 0.0f;
#pragma unroll
  for (int q = 0; q < NN; ++q) modes[q] = in[q] * inv;
}

// Modes of rho*p of element e (one thread per element).
template <int D, int N, typename TS>
__device__ __forceinline__ void element_modes(const FeatParams& P, const TS* __restrict__ u,
                                              int64_t e, float* modes, float& energy,
                                              bool& positive) {
  constexpr int NN = Pow<N, D>::value;
  float a[NN];
#pragma unroll
  for (int q = 0; q < NN; ++q) a[q] = node_rho_p<D, TS>(P, u, e * NN + q);
  modes_from_rho_p<D, N>(P, a, modes, energy, positive);
}

// HG logistic of an energy indicator, clipped (indicators_2d.jl:92-100)
__device__ __forceinline__ float hg_logistic(float energy, float thr, float s_par, float alpha_min,
                                             float alpha_max) {
  float al = 1.0f / (1.0f + expf(-s_par / thr * (energy - thr)));
  if (al < alpha_min) al = 0.0f;
  if (al > 1.0f - alpha_min) al = 1.0f;
  return fminf(alpha_max, al);
}

template <int D, int N, typename TS>
__global__ void features_kernel(const FeatParams P, const TS* __restrict__ u,
                                float* __restrict__ feat, float* __restrict__ target,
                                float* __restrict__ alpha_hg, int32_t* __restrict__ pos_flag) {
  constexpr int NN = Pow<N, D>::value;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.E) return;
  float m[NN], energy;
  bool positive;
  element_modes<D, N, TS>(P, u, e, m, energy, positive);
  alpha_hg[e] = hg_logistic(energy, P.hg_threshold, P.hg_parameter_s, P.alpha_min, P.alpha_max);
#pragma unroll
  for (int q = 0; q < NN; ++q) feat[(size_t)e * NN + q] = m[q];
  if (target) target[e] = sqrtf(fmaxf(energy, 0.0f));
  pos_flag[e] = positive ? 0 : 2;
}

// ---------------------------------------------------------------------------
// The network on the 5th-generation tensor cores (tcgen05), for deployment
// (features computed from the state, blending factor out) and for predictions
// of explicit rows.  A block of 128 threads walks tiles of 128 elements, one
// thread per element, i.e. per row of the MMA operands and per TMEM lane:
//   layer 1  D = X W1^T: X [128 x K1] (the n^d features, zero-padded to K1, a
//            multiple of 16), W1 [H x K1]; FP32 accumulators in TMEM;
//   layer 2  D = relu(D + b1) W2^T, in the same TMEM columns;
//   output   b3 + sum_j w3_j relu(D_j + b2_j) in FP32 on the CUDA cores, from
//            the thread's own TMEM lane.
// The weights are BF16 (exact MMA operands).  Each FP32 layer input x is fed
// as two BF16 operands, hi = bf16(x) and lo = bf16(x - hi), multiplied by the
// same weights into the same accumulator: the products are exact and x is
// represented to about 2^-17, so the tensor cores evaluate the FP32 network
// the training kernel fits (a plain BF16 rounding of the inputs, 2^-9, would
// erase the small high-mode part of the features next to the mean mode).
// One thread issues the MMAs (M = 128, N = H, K = 16 per instruction) and
// commits them to an mbarrier that every thread waits on; the layer inputs are
// written to shared memory by all threads in the K-major layout of
// tg_tcgen05.cuh, and the weights arrive once per block, already in that
// layout, by bulk copies of the weight image (mlp_weight_image_kernel).  The layer-2 operands overlay
// the layer-1 ones (layer 1 has completed when they are written).  The same
// code serves both entry points, so deployed predictions and tg_mlp_predict
// agree bit for bit.
// ---------------------------------------------------------------------------
struct AlphaParams {
  float sqrt_thr, band, thr, s_par, alpha_min, alpha_max;
};

// Status bit set when a wait for the tensor core gave up (the block stops).
constexpr int32_t STATUS_TC_TIMEOUT = 4;
constexpr uint32_t TC_WAIT_POLLS = 1u << 22;

template <int NM, int H>
struct TcShape {
  static constexpr int ROWS = 128;
  static constexpr int K1 = (NM + 15) / 16 * 16;
  static constexpr int OW1 = 0;
  static constexpr int OW2 = OW1 + H * K1 * 2;
  static constexpr int OA = OW2 + H * H * 2;            // operand area
  static constexpr int A1 = ROWS * K1 * 2, A2 = ROWS * H * 2;  // bytes of one hi or lo operand
  static constexpr int OA1H = OA, OA1L = OA + A1;       // layer 1: hi, lo
  static constexpr int OA2H = OA, OA2L = OA + A2;       // layer 2: hi, lo (overlay layer 1)
  static constexpr int OVEC = OA + 2 * (A1 > A2 ? A1 : A2);  // b1[H], b2[H], w3[H], b3 (FP32)
  // the deployment stages rho*p of the tile's nodes ([ROWS][NM + 1] floats)
  // in the operand area before the layer-1 operands are written
  static_assert(ROWS * (NM + 1) * 4 <= OVEC - OA, "rho*p staging fits the operand area");
  // the weight image (mlp_weight_image_kernel): W1 and W2 in their operand
  // layouts (bytes [OW1, OA)), then the FP32 vectors padded to 16 bytes; two
  // bulk copies per block
  static constexpr int WIMG = OA - OW1;
  static constexpr int VIMG = (3 * H + 4) * 4;
  static_assert(WIMG % 16 == 0 && VIMG % 16 == 0 && OVEC % 16 == 0, "bulk copy sizes");
  static constexpr int OBAR = OVEC + VIMG;              // mbarriers: MMA, staging, weights
  static constexpr int OSLOT = OBAR + 24;               // TMEM base address
  // 2D deployment: the tile's state (n^d nodes x 4 values, float-float or
  // FP64: 32 bytes per node), staged by one bulk copy per tile
  static constexpr int STAGE_BYTES = ROWS * NM * 32;
  static constexpr int OSTG = (OSLOT + 8 + 127) / 128 * 128;
  static constexpr int SMEM_STAGED = OSTG + STAGE_BYTES;
  // deployment from rho*p rows (the stage kernel's output): NM floats per element
  static constexpr int SMEM_RP = OSTG + ROWS * NM * 4;
  static constexpr int SMEM = OSLOT + 8;
  static constexpr int TCOLS = H;                       // layer 2 reuses layer 1's columns
  static constexpr uint32_t IDESC = tc::idesc_bf16_f32(ROWS, H);
  static_assert(OBAR % 8 == 0, "mbarrier alignment");
  static_assert(H == 64 || H == 128, "TMEM columns: a power of two >= 32");
};

// 8 FP32 values as BF16 hi and lo parts (v = hi + lo + O(2^-17 |v|)).
__device__ __forceinline__ void split8_bf16(const float* v, uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int j = 0; j < 8; j += 2) {
    const __nv_bfloat162 bh = __floats2bfloat162_rn(v[j], v[j + 1]);
    const float2 fh = __bfloat1622float2(bh);
    const __nv_bfloat162 bl = __floats2bfloat162_rn(v[j] - fh.x, v[j + 1] - fh.y);
    h[j / 2] = *reinterpret_cast<const uint32_t*>(&bh);
    l[j / 2] = *reinterpret_cast<const uint32_t*>(&bl);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Row r of the hi and lo K-major operands with K columns from FP32 values
// (columns beyond `n` are zero): 16-byte stores of 8 values.
template <int K>
__device__ __forceinline__ void store_row_split(unsigned char* hi, unsigned char* lo, int r,
                                                const float* v, int n) {
#pragma unroll
  for (int c = 0; c < K; c += 8) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = c + j < n ? v[c + j] : 0.0f;
    uint4 h, l;
    split8_bf16(x, h, l);
    const int o = tc::kmajor_offset(r, c, K);
    *reinterpret_cast<uint4*>(hi + o) = h;
    *reinterpret_cast<uint4*>(lo + o) = l;
  }
}

// SRC 0: features of the elements of the state u (deployment: blending
// factors with the HG fallback, per-element report); SRC 1: rows of x
// ([nrows][NM], predictions only); SRC 2: deployment as SRC 0 from x = rho*p
// of the state's nodes ([E][NM], written by the previous stage kernel), the
// same features without reading the state.
template <int D, int N, int NM, int H, int SRC, typename TS, typename R>
__global__ void __launch_bounds__(128) mlp_tc_kernel(
    const FeatParams P, const TS* __restrict__ u, const float* __restrict__ x, int64_t nrows,
    const unsigned char* __restrict__ wimg, const AlphaParams A, R* __restrict__ alpha_raw,
    float* __restrict__ pred_out, float* __restrict__ hg_out, int32_t* __restrict__ flag_out,
    unsigned long long* __restrict__ stats, int32_t* __restrict__ status) {
  using S = TcShape<NM, H>;
  constexpr int K1 = S::K1;
  extern __shared__ __align__(128) unsigned char tc_smem[];
  unsigned char* sm = tc_smem;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S::OBAR);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + S::OSLOT);
  float* s_b1 = reinterpret_cast<float*>(sm + S::OVEC);
  float* s_b2 = s_b1 + H;
  float* s_w3 = s_b2 + H;  // s_w3[H] = b3
  // 2D deployment stages each tile's state with one bulk copy (contiguous in
  // the element order), the next tile's issued as soon as this one's rho*p
  // has been read
  constexpr bool STAGED = (SRC == 0 && D == 2) || SRC == 2;
  constexpr int NODE_BYTES = SRC == 2 ? 4 : 32;  // staged bytes per node
  // rho*p rows of 16-byte multiples are read by each thread straight from the
  // staging buffer (four-way bank conflicts, against a re-layout pass); up to
  // 16 values, where the registers allow it
  constexpr bool DIRECT_ROWS = SRC == 2 && NM % 4 == 0 && NM <= 16;
  uint64_t* sbar = bar + 1;
  uint64_t* wbar = bar + 2;
  float4* s_stg = reinterpret_cast<float4*>(sm + S::OSTG);
  const int64_t total = SRC == 1 ? nrows : P.E;
  const int64_t ntiles = (total + S::ROWS - 1) / S::ROWS;
  const unsigned char* stage_src =
      SRC == 2 ? reinterpret_cast<const unsigned char*>(x) : reinterpret_cast<const unsigned char*>(u);
  auto issue_tile = [&](int64_t t) {  // one thread
    const int64_t rows = min((int64_t)S::ROWS, total - t * S::ROWS);
    const uint32_t bytes = (uint32_t)(rows * NM * NODE_BYTES);
    tc::mbar_arrive_expect_tx(sbar, bytes);
    tc::bulk_g2s(s_stg, stage_src + (size_t)t * S::ROWS * NM * NODE_BYTES, bytes, sbar);
  };

  // the first tile's staging and the weight image, by bulk copies
  if (tid == 0) {
    tc::mbar_init(bar, 1);
    tc::mbar_init(wbar, 1);
    if (STAGED) tc::mbar_init(sbar, 1);
    tc::fence_mbar_init();
    if (STAGED && blockIdx.x < ntiles) issue_tile(blockIdx.x);
    tc::mbar_arrive_expect_tx(wbar, S::WIMG + S::VIMG);
    tc::bulk_g2s(sm + S::OW1, wimg, S::WIMG, wbar);
    tc::bulk_g2s(sm + S::OVEC, wimg + S::WIMG, S::VIMG, wbar);
  }
  if (warp == 0) {
    tc::tmem_alloc(slot, S::TCOLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
  const uint32_t a1h = tc::smem_u32(sm + S::OA1H), a1l = tc::smem_u32(sm + S::OA1L);
  const uint32_t a2h = tc::smem_u32(sm + S::OA2H), a2l = tc::smem_u32(sm + S::OA2L);
  const uint32_t w1 = tc::smem_u32(sm + S::OW1), w2 = tc::smem_u32(sm + S::OW2);
  if (SRC != 1 && blockIdx.x == 0 && tid == 0) atomicAdd(&stats[0], (unsigned long long)P.E);

  uint32_t phase = 0, sphase = 0;
  bool mma_in_flight = false, staging_in_flight = STAGED && blockIdx.x < ntiles;
  bool failed = __syncthreads_or(!tc::mbar_wait_bounded(wbar, 0, TC_WAIT_POLLS));
  const bool weights_late = failed;
  for (int64_t tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
    const int64_t e = tile * S::ROWS + tid;
    const bool act = e < total;
    float xv[NM];
    float energy = 0.0f;
    bool positive = true;
    if constexpr (SRC != 1) {
      // rho*p of the tile's nodes, one node per thread and pass, so that a
      // warp's loads are consecutive nodes; staged in the (free) operand area
      float* s_rp = reinterpret_cast<float*>(sm + S::OA);
      const int64_t n0 = tile * S::ROWS * NM;
      const int64_t nn = (min(total, (tile + 1) * S::ROWS) - tile * S::ROWS) * NM;
      float a[NM];
      if constexpr (STAGED) {
        if (__syncthreads_or(!tc::mbar_wait_bounded(sbar, sphase, TC_WAIT_POLLS))) {
          failed = true;
          break;
        }
        sphase ^= 1;
        staging_in_flight = false;
        if constexpr (DIRECT_ROWS) {
          if (act) {
            const float4* row = s_stg + tid * (NM / 4);
#pragma unroll
            for (int q = 0; q < NM / 4; ++q) {
              const float4 f = row[q];
              a[4 * q] = f.x;
              a[4 * q + 1] = f.y;
              a[4 * q + 2] = f.z;
              a[4 * q + 3] = f.w;
            }
          }
        } else {
#pragma unroll 4
          for (int j = 0; j < NM; ++j) {
            const int k = j * S::ROWS + tid;
            if (k < nn)
              s_rp[(k / NM) * (NM + 1) + k % NM] =
                  SRC == 2 ? reinterpret_cast<const float*>(s_stg)[k] : staged_rho_p<TS>(P, s_stg, k);
          }
        }
        __syncthreads();
        // the staging buffer is free: the next tile's state lands meanwhile
        if (tile + gridDim.x < ntiles) {
          if (tid == 0) {
            tc::fence_proxy_async_smem();  // the reads above before the copy's writes
            issue_tile(tile + gridDim.x);
          }
          staging_in_flight = true;
        }
      } else {
#pragma unroll 4
        for (int j = 0; j < NM; ++j) {
          const int k = j * S::ROWS + tid;
          if (k < nn) s_rp[(k / NM) * (NM + 1) + k % NM] = node_rho_p<D, TS>(P, u, n0 + k);
        }
        __syncthreads();
      }
      if (act) {
        if constexpr (!DIRECT_ROWS) {
#pragma unroll
          for (int q = 0; q < NM; ++q) a[q] = s_rp[tid * (NM + 1) + q];
        }
        modes_from_rho_p<D, N>(P, a, xv, energy, positive);
      } else {
#pragma unroll
        for (int k = 0; k < NM; ++k) xv[k] = 0.0f;
      }
      __syncthreads();  // all rows read before the operand area is written
    } else {
#pragma unroll
      for (int k = 0; k < NM; ++k) xv[k] = act ? x[e * NM + k] : 0.0f;
    }
    store_row_split<K1>(sm + S::OA1H, sm + S::OA1L, tid, xv, NM);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < K1 / 16; ++s) {
        const uint64_t b = tc::smem_desc(w1 + s * 256, 128, K1 * 16);
        tc::mma_bf16(tmem, tc::smem_desc(a1h + s * 256, 128, K1 * 16), b, S::IDESC, s > 0);
        tc::mma_bf16(tmem, tc::smem_desc(a1l + s * 256, 128, K1 * 16), b, S::IDESC, 1);
      }
      tc::commit(bar);
    }
    if (__syncthreads_or(!tc::mbar_wait_bounded(bar, phase, TC_WAIT_POLLS))) {
      failed = mma_in_flight = true;
      break;
    }
    phase ^= 1;
    tc::fence_after_sync();
    // layer 1 epilogue: bias, ReLU -> row tid of the layer-2 operands (hi, lo)
#pragma unroll
    for (int c0 = 0; c0 < H; c0 += 32) {
      float v[32];
      tc::tmem_ld32(trow + c0, v);
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        const float4 b = *reinterpret_cast<const float4*>(s_b1 + c0 + j);
        v[j] = fmaxf(v[j] + b.x, 0.0f);
        v[j + 1] = fmaxf(v[j + 1] + b.y, 0.0f);
        v[j + 2] = fmaxf(v[j + 2] + b.z, 0.0f);
        v[j + 3] = fmaxf(v[j + 3] + b.w, 0.0f);
      }
#pragma unroll
      for (int g = 0; g < 32; g += 8) {
        uint4 h, l;
        split8_bf16(v + g, h, l);
        const int o = tc::kmajor_offset(tid, c0 + g, H);
        *reinterpret_cast<uint4*>(sm + S::OA2H + o) = h;
        *reinterpret_cast<uint4*>(sm + S::OA2L + o) = l;
      }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int s = 0; s < H / 16; ++s) {
        const uint64_t b = tc::smem_desc(w2 + s * 256, 128, H * 16);
        tc::mma_bf16(tmem, tc::smem_desc(a2h + s * 256, 128, H * 16), b, S::IDESC, s > 0);
        tc::mma_bf16(tmem, tc::smem_desc(a2l + s * 256, 128, H * 16), b, S::IDESC, 1);
      }
      tc::commit(bar);
    }
    if (__syncthreads_or(!tc::mbar_wait_bounded(bar, phase, TC_WAIT_POLLS))) {
      failed = mma_in_flight = true;
      break;
    }
    phase ^= 1;
    tc::fence_after_sync();
    // output layer from this thread's TMEM lane
    float out = s_w3[H];
#pragma unroll
    for (int c0 = 0; c0 < H; c0 += 32) {
      float v[32];
      tc::tmem_ld32(trow + c0, v);
#pragma unroll
      for (int j = 0; j < 32; j += 4) {
        const float4 b = *reinterpret_cast<const float4*>(s_b2 + c0 + j);
        const float4 wv = *reinterpret_cast<const float4*>(s_w3 + c0 + j);
        out = fmaf(wv.x, fmaxf(v[j] + b.x, 0.0f), out);
        out = fmaf(wv.y, fmaxf(v[j + 1] + b.y, 0.0f), out);
        out = fmaf(wv.z, fmaxf(v[j + 2] + b.z, 0.0f), out);
        out = fmaf(wv.w, fmaxf(v[j + 3] + b.w, 0.0f), out);
      }
    }
    tc::fence_before_sync();  // the next tile's MMAs are issued after a barrier
    if constexpr (SRC == 1) {
      if (act) pred_out[e] = out;
    } else {
      // blending factor: the network's, or HG's near the switch and for
      // non-positive rho*p; then the clipping of indicators_2d.jl:92-100
      const float hg = hg_logistic(energy, A.thr, A.s_par, 0.0f, 1.0f);
      int f = positive ? 0 : 2;
      if (f == 0 && !(fabsf(out - A.sqrt_thr) >= A.band)) f = 1;  // also catches NaN
      const float ep = fmaxf(out, 0.0f);
      float al = f != 0 ? hg : 1.0f / (1.0f + expf(-A.s_par / A.thr * (ep * ep - A.thr)));
      if (al < A.alpha_min) al = 0.0f;
      if (al > 1.0f - A.alpha_min) al = 1.0f;
      al = fminf(A.alpha_max, al);
      const unsigned nb1 = __popc(__ballot_sync(0xffffffffu, act && f == 1));
      const unsigned nb2 = __popc(__ballot_sync(0xffffffffu, act && f == 2));
      if (lane == 0 && nb1) atomicAdd(&stats[1], (unsigned long long)nb1);
      if (lane == 0 && nb2) atomicAdd(&stats[2], (unsigned long long)nb2);
      if (act) {
        alpha_raw[e] = (R)al;
        pred_out[e] = out;
        hg_out[e] = hg;
        flag_out[e] = f;
      }
    }
  }
  if (failed) {
    // a wait gave up: report it, wait (bounded) for the MMAs or the staging
    // copy still in flight, then free the tensor memory as on the normal path
    if (tid == 0) atomicOr(status, STATUS_TC_TIMEOUT);
    if (mma_in_flight) tc::mbar_wait_bounded(bar, phase, TC_WAIT_POLLS);
    if (staging_in_flight) tc::mbar_wait_bounded(sbar, sphase, TC_WAIT_POLLS);
    if (weights_late) tc::mbar_wait_bounded(wbar, 0, TC_WAIT_POLLS);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, S::TCOLS);
  }
}

// ---------------------------------------------------------------------------
// Training: fused forward + backward over a tile of TS samples (one thread
// per sample), weight gradients as tile-level contractions written as one
// partial sum per block and tile squared error; reduce_partials_kernel sums
// them in block order, so training is reproducible bit for bit.  Loss: mean
// squared error.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}

template <int NM, int H, int TS>
__global__ void __launch_bounds__(TS) mlp_train_kernel(const __nv_bfloat16* __restrict__ w,
                                                       const float* __restrict__ X,
                                                       const float* __restrict__ Y, int64_t M,
                                                       const int64_t* __restrict__ idx_explicit,
                                                       uint64_t seed, int batch, int holdout,
                                                       float* __restrict__ grad,
                                                       float* __restrict__ loss) {
  // grad: [gridDim.x][nparams] partial sums, loss: [gridDim.x] squared errors
  extern __shared__ float sm[];
  float* sX = sm;             // [NM][TS]
  float* sH1 = sX + NM * TS;  // [H][TS]: h1, later dz1
  float* sH2 = sH1 + H * TS;  // [H][TS]: h2, later dz2
  float* sD = sH2 + H * TS;   // [TS]: dout
  const MlpLayout L{NM, H};
  const int tid = threadIdx.x;
  const int k0 = blockIdx.x * TS + tid;
  const bool act = k0 < batch;
  int64_t s = 0;
  if (act) {
    if (idx_explicit) {
      s = idx_explicit[k0];
    } else {
      // sample with replacement among the training rows (every holdout-th row is held out)
      s = (int64_t)(hash32(seed * 0x9e3779b97f4a7c15ull + (uint64_t)k0) % (uint32_t)M);
      if (holdout > 1 && s % holdout == 0) s = (s + 1) % M;
    }
  }
  for (int k = 0; k < NM; ++k) sX[k * TS + tid] = act ? X[s * NM + k] : 0.0f;
  for (int i = 0; i < H; ++i) {
    float z = wld(w, L.b1() + i);
    for (int k = 0; k < NM; ++k) z = fmaf(wld(w, L.w1() + i * NM + k), sX[k * TS + tid], z);
    sH1[i * TS + tid] = fmaxf(z, 0.0f);
  }
  float out = wld(w, L.b3());
  for (int i = 0; i < H; ++i) {
    float z = wld(w, L.b2() + i);
    for (int j = 0; j < H; ++j) z = fmaf(wld(w, L.w2() + i * H + j), sH1[j * TS + tid], z);
    const float h = fmaxf(z, 0.0f);
    sH2[i * TS + tid] = h;
    out = fmaf(wld(w, L.w3() + i), h, out);
  }
  const float r = act ? out - Y[s] : 0.0f;
  sD[tid] = act ? 2.0f * r / (float)batch : 0.0f;
  __syncthreads();
  if (tid == 0) {
    // squared error of the tile, summed in a fixed order (from the residuals)
    float l = 0;
    for (int t = 0; t < TS; ++t) {
      const float rt = sD[t] * (0.5f * (float)batch);
      l = fmaf(rt, rt, l);
    }
    loss[blockIdx.x] = l;
  }
  // this block's gradient partial sums: grad[blockIdx.x][k]
  grad += (size_t)blockIdx.x * L.count();
  // output layer gradients
  for (int i = tid; i < H; i += TS) {
    float g = 0;
    for (int t = 0; t < TS; ++t) g = fmaf(sD[t], sH2[i * TS + t], g);
    grad[L.w3() + i] = g;
  }
  if (tid == 0) {
    float g = 0;
    for (int t = 0; t < TS; ++t) g += sD[t];
    grad[L.b3()] = g;
  }
  __syncthreads();
  // dz2 = dout * w3 * [h2 > 0]   (in place of h2)
  for (int i = 0; i < H; ++i) {
    const float h = sH2[i * TS + tid];
    sH2[i * TS + tid] = h > 0.0f ? sD[tid] * wld(w, L.w3() + i) : 0.0f;
  }
  __syncthreads();
  // dW2[i][j] = sum_t dz2[i][t] h1[j][t], db2[i] = sum_t dz2[i][t]
  for (int i = tid; i < H; i += TS) {
    float gb = 0;
    for (int t = 0; t < TS; ++t) gb += sH2[i * TS + t];
    grad[L.b2() + i] = gb;
    for (int j = 0; j < H; ++j) {
      float g = 0;
      for (int t = 0; t < TS; ++t) g = fmaf(sH2[i * TS + t], sH1[j * TS + t], g);
      grad[L.w2() + i * H + j] = g;
    }
  }
  __syncthreads();
  // dh1[j] = sum_i dz2[i] W2[i][j]; dz1 = dh1 [h1 > 0]  (own sample, in place of h1)
  {
    float dh[H];
    for (int j = 0; j < H; ++j) dh[j] = 0.0f;
    for (int i = 0; i < H; ++i) {
      const float dz = sH2[i * TS + tid];
      if (dz != 0.0f)
        for (int j = 0; j < H; ++j) dh[j] = fmaf(dz, wld(w, L.w2() + i * H + j), dh[j]);
    }
    __syncthreads();
    for (int j = 0; j < H; ++j) sH1[j * TS + tid] = sH1[j * TS + tid] > 0.0f ? dh[j] : 0.0f;
  }
  __syncthreads();
  // dW1[i][k] = sum_t dz1[i][t] x[k][t], db1[i] = sum_t dz1[i][t]
  for (int i = tid; i < H; i += TS) {
    float gb = 0;
    for (int t = 0; t < TS; ++t) gb += sH1[i * TS + t];
    grad[L.b1() + i] = gb;
    for (int k = 0; k < NM; ++k) {
      float g = 0;
      for (int t = 0; t < TS; ++t) g = fmaf(sH1[i * TS + t], sX[k * TS + t], g);
      grad[L.w1() + i * NM + k] = g;
    }
  }
}

// Sums of the per-block partials in block order (deterministic): the
// gradient, and the tiles' squared errors added to loss[0] (with the sample
// count in loss[1]).
__global__ void reduce_partials_kernel(const float* __restrict__ part, int nblk, int64_t n,
                                       float* __restrict__ grad, const float* __restrict__ lpart,
                                       float* __restrict__ loss, int batch) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) {
    float g = 0;
    for (int b = 0; b < nblk; ++b) g += part[(size_t)b * n + k];
    grad[k] = g;
  }
  if (k == 0) {
    float l = 0;
    for (int b = 0; b < nblk; ++b) l += lpart[b];
    loss[0] += l;
    loss[1] += (float)batch;
  }
}

__global__ void adam_kernel(float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                            float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.0f - b1) * gk;
  const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float wk = w[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  w[k] = wk;
  wb[k] = __float2bfloat16(wk);
  g[k] = 0.0f;
}

__global__ void to_bf16_kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                               int64_t n) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) wb[k] = __float2bfloat16(w[k]);
}

// The weight image that every block of mlp_tc_kernel copies into shared
// memory: W1 [H][NM] zero-padded to K1 columns and W2 [H][H], BF16, in the
// K-major operand layouts, then b1, b2, w3 and b3 as FP32, zero-padded to a
// multiple of 16 bytes ((3H + 4) floats).
__global__ void mlp_weight_image_kernel(const __nv_bfloat16* __restrict__ w, MlpLayout L, int K1,
                                        unsigned char* __restrict__ img) {
  const int NM = L.NM, H = L.H;
  const int n1 = H * K1, n2 = H * H, nv = 3 * H + 4;
  unsigned char* w2img = img + (size_t)H * K1 * 2;
  float* vimg = reinterpret_cast<float*>(w2img + (size_t)H * H * 2);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n1 + n2 + nv;
       k += gridDim.x * blockDim.x) {
    if (k < n1) {
      const int i = k / K1, j = k - i * K1;
      *reinterpret_cast<__nv_bfloat16*>(img + tc::kmajor_offset(i, j, K1)) =
          j < NM ? w[L.w1() + i * NM + j] : __float2bfloat16(0.0f);
    } else if (k < n1 + n2) {
      const int q = k - n1, i = q / H, j = q - i * H;
      *reinterpret_cast<__nv_bfloat16*>(w2img + tc::kmajor_offset(i, j, H)) = w[L.w2() + q];
    } else {
      const int q = k - n1 - n2;
      float v = 0.0f;
      if (q < H) v = __bfloat162float(w[L.b1() + q]);
      else if (q < 2 * H) v = __bfloat162float(w[L.b2() + q - H]);
      else if (q < 3 * H) v = __bfloat162float(w[L.w3() + q - 2 * H]);
      else if (q == 3 * H) v = __bfloat162float(w[L.b3()]);
      vimg[q] = v;
    }
  }
}

}  // namespace tg

using namespace tg;

static int mfail(tg_mlp* m, int code, const char* msg) {
  if (m) m->err = msg;
  set_thread_error(msg);
  return code;
}

#define MCUDA(m, call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return mfail((m), TG_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

static int launch_features(tg_mlp* m, tg_ctx* c, float* feat, float* target, float* alpha_hg,
                           int32_t* flag, cudaStream_t* s_out, int64_t* E_out) {
  const void* state;
  int ff, D, N;
  int64_t E;
  double gamma;
  const double* vinv;
  void* stream;
  int rc = ctx_state_view(c, &state, &ff, &D, &N, &E, &gamma, &vinv, &stream);
  if (rc) return rc;
  if (D != m->D || N != m->N) return mfail(m, TG_ERR_INVALID_ARGUMENT, "network/context shape mismatch");
  FeatParams P{};
  P.E = E;
  P.gamma = gamma;
  for (int k = 0; k < N * N; ++k) P.Vinv[k] = (float)vinv[k];
  // HG constants of this polydeg (indicators.jl:128-131)
  P.hg_threshold = (float)(0.5 * std::pow(10.0, -1.8 * std::pow((double)N, 0.25)));
  P.hg_parameter_s = (float)std::log((1 - 0.0001) / 0.0001);
  P.alpha_min = 0.0f;
  P.alpha_max = 1.0f;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned nb = (unsigned)((E + 127) / 128);
#define FEAT(DD, NN)                                                                           \
  if (D == DD && N == NN) {                                                                    \
    if (ff)                                                                                    \
      features_kernel<DD, NN, float2><<<nb, 128, 0, s>>>(P, (const float2*)state, feat, target, \
                                                         alpha_hg, flag);                      \
    else                                                                                       \
      features_kernel<DD, NN, double><<<nb, 128, 0, s>>>(P, (const double*)state, feat, target, \
                                                         alpha_hg, flag);                      \
  } else
  FEAT(2, 3) FEAT(2, 4) FEAT(2, 5) FEAT(3, 3) FEAT(3, 4) {
    return mfail(m, TG_ERR_UNSUPPORTED, "learned indicator: polydeg 2..4 only");
  }
#undef FEAT
  MCUDA(m, cudaGetLastError());
  *s_out = s;
  *E_out = E;
  return TG_OK;
}

// One launch of the tensor-core MLP kernel: a persistent grid of at most as
// many 128-thread blocks as fit on the GPU at once (shared memory, registers
// and tensor memory: 512 TMEM columns per SM).
template <int D, int N, int NM, int H, int SRC, typename TS, typename R>
static int launch_tc(tg_mlp* m, const FeatParams& P, const TS* u, const float* x, int64_t rows,
                     const AlphaParams& A, R* alpha_raw, float* pred, int32_t* status,
                     cudaStream_t s) {
  using S = TcShape<NM, H>;
  auto kern = mlp_tc_kernel<D, N, NM, H, SRC, TS, R>;
  constexpr int SMEM = SRC == 2 ? S::SMEM_RP : ((SRC == 0 && D == 2) ? S::SMEM_STAGED : S::SMEM);
  static int resident[64] = {0};  // blocks per SM, per device
  int dev = 0;
  MCUDA(m, cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return mfail(m, TG_ERR_UNSUPPORTED, "device index");
  if (resident[dev] == 0) {
    MCUDA(m, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM));
    MCUDA(m, cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
    // Blocks per SM from the kernel's own resources: registers, shared memory
    // (plus the 1 KB the driver reserves per block) and tensor memory (512
    // columns per SM).  The runtime's occupancy query reports one block per
    // SM for this kernel, which would leave most of the GPU idle.
    cudaFuncAttributes fa{};
    MCUDA(m, cudaFuncGetAttributes(&fa, kern));
    int smem_sm = 0, regs_sm = 0;
    MCUDA(m, cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    MCUDA(m, cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    const int regs = (std::max(fa.numRegs, 1) + 7) / 8 * 8;  // allocated in units of 8
    const int by_regs = regs_sm / (regs * S::ROWS);
    const int by_smem = smem_sm / (SMEM + 1024);
    resident[dev] = std::max(1, std::min({by_regs, by_smem, 512 / S::TCOLS, 2048 / S::ROWS}));
  }
  int sms = 0;
  MCUDA(m, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t ntiles = (rows + S::ROWS - 1) / S::ROWS;
  if (ntiles == 0) return TG_OK;
  const unsigned nb = (unsigned)std::min<int64_t>(ntiles, (int64_t)sms * resident[dev]);
  if (m->wimg_bytes != (size_t)(S::WIMG + S::VIMG))
    return mfail(m, TG_ERR_INVALID_ARGUMENT, "weight image of another network shape");
  kern<<<nb, S::ROWS, SMEM, s>>>(P, u, x, rows, m->d_wimg, A, alpha_raw, pred, m->d_hg,
                                    m->d_flag, m->d_stats, status);
  MCUDA(m, cudaGetLastError());
  return TG_OK;
}

// Predictions for rows x [M][NM] (device) into pred [M] (device).
static int launch_predict(tg_mlp* m, const float* x, int64_t M, float* pred, cudaStream_t s) {
  FeatParams P{};
  AlphaParams A{};
#define PRED(DD, NN, NMv, Hv)                                                              \
  if (m->D == DD && m->N == NN)                                                            \
    return launch_tc<DD, NN, NMv, Hv, 1, float, float>(m, P, nullptr, x, M, A, nullptr, pred, \
                                                       m->d_status, s);
  PRED(2, 3, 9, 64)
  PRED(2, 4, 16, 64)
  PRED(2, 5, 25, 64)
  PRED(3, 3, 27, 128)
  PRED(3, 4, 64, 128)
#undef PRED
  return mfail(m, TG_ERR_UNSUPPORTED, "network shape not compiled");
}

namespace tg {
int32_t* ctx_status_word(tg_ctx* c);
const float* ctx_state_rho_p(tg_ctx* c);

// Called by the context before every stage when the learned indicator is on:
// writes the blending factors (unsmoothed) into alpha_raw (R = float for mixed
// contexts, double for FP64 ones), one tensor-core kernel per stage.
int mlp_alpha(tg_mlp* m, tg_ctx* c, void* alpha_raw, bool fp64, float alpha_min,
              float alpha_max) {
  if (m->ecap == 0) return mfail(m, TG_ERR_STATE, "learned indicator not prepared for this context");
  const void* state;
  int ff, D, N;
  int64_t E;
  double gamma;
  const double* vinv;
  void* stream;
  int rc = ctx_state_view(c, &state, &ff, &D, &N, &E, &gamma, &vinv, &stream);
  if (rc) return rc;
  if (D != m->D || N != m->N) return mfail(m, TG_ERR_INVALID_ARGUMENT, "network/context shape mismatch");
  if (E > m->ecap) return mfail(m, TG_ERR_STATE, "context larger than prepared");
  FeatParams P{};
  P.E = E;
  P.gamma = gamma;
  for (int k = 0; k < N * N; ++k) P.Vinv[k] = (float)vinv[k];
  AlphaParams A{};
  // HG constants of this polydeg (indicators.jl:128-131)
  A.thr = (float)(0.5 * std::pow(10.0, -1.8 * std::pow((double)N, 0.25)));
  A.s_par = (float)std::log((1 - 0.0001) / 0.0001);
  A.sqrt_thr = (float)m->sqrt_threshold;
  A.band = m->band;
  A.alpha_min = alpha_min;
  A.alpha_max = alpha_max;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t* status = ctx_status_word(c);
  // rho*p of the state from the previous stage kernel, when the context keeps it
  const float* rp = ctx_state_rho_p(c);
#define DEPLOY(DD, NN, NMv, Hv)                                                                 \
  if (D == DD && N == NN) {                                                                     \
    if (ff && rp && DD == 2)                                                                    \
      return launch_tc<DD, NN, NMv, Hv, 2, float2, float>(                                      \
          m, P, nullptr, rp, E, A, (float*)alpha_raw, m->d_pred, status, s);                    \
    if (ff)                                                                                     \
      return launch_tc<DD, NN, NMv, Hv, 0, float2, float>(                                      \
          m, P, (const float2*)state, nullptr, E, A, (float*)alpha_raw, m->d_pred, status, s);  \
    return launch_tc<DD, NN, NMv, Hv, 0, double, double>(                                       \
        m, P, (const double*)state, nullptr, E, A, (double*)alpha_raw, m->d_pred, status, s);   \
  }
  DEPLOY(2, 3, 9, 64)
  DEPLOY(2, 4, 16, 64)
  DEPLOY(2, 5, 25, 64)
  DEPLOY(3, 3, 27, 128)
  DEPLOY(3, 4, 64, 128)
#undef DEPLOY
  (void)fp64;
  return mfail(m, TG_ERR_UNSUPPORTED, "learned indicator: polydeg 2..4 only");
}
}  // namespace tg

// Partial-sum buffers for `nblk` training blocks (grown on demand).
static int ensure_partials(tg_mlp* m, int64_t nblk) {
  if (nblk <= m->part_blocks) return TG_OK;
  cudaFree(m->d_gpart);
  cudaFree(m->d_lpart);
  m->d_gpart = m->d_lpart = nullptr;
  m->part_blocks = 0;
  MCUDA(m, cudaMalloc(&m->d_gpart, sizeof(float) * nblk * m->nparams));
  MCUDA(m, cudaMalloc(&m->d_lpart, sizeof(float) * nblk));
  m->part_blocks = nblk;
  return TG_OK;
}

// One forward + backward pass over `batch` rows (explicit indices `idx`, or
// drawn from the training set by `seed`): gradient into d_g, squared error and
// sample count added to d_loss.
static int train_pass(tg_mlp* m, const float* X, const float* Y, int64_t M, const int64_t* idx,
                      uint64_t seed, int batch, int holdout) {
  constexpr int TS = 64;
  const int nb = (batch + TS - 1) / TS;
  int rc = ensure_partials(m, nb);
  if (rc) return rc;
  const size_t smem = sizeof(float) * (m->NM * TS + 2 * m->H * TS + TS);
#define TRAIN(NMv, Hv)                                                                            \
  if (m->NM == NMv && m->H == Hv) {                                                               \
    MCUDA(m, cudaFuncSetAttribute(mlp_train_kernel<NMv, Hv, TS>,                                  \
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));       \
    mlp_train_kernel<NMv, Hv, TS><<<nb, TS, smem>>>(m->d_wb, X, Y, M, idx, seed, batch, holdout,  \
                                                    m->d_gpart, m->d_lpart);                       \
  } else
  TRAIN(16, 64) TRAIN(9, 64) TRAIN(25, 64) TRAIN(27, 128) TRAIN(64, 128) {
    return mfail(m, TG_ERR_UNSUPPORTED, "network shape not compiled");
  }
#undef TRAIN
  reduce_partials_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(
      m->d_gpart, nb, m->nparams, m->d_g, m->d_lpart, m->d_loss, batch);
  MCUDA(m, cudaGetLastError());
  return TG_OK;
}

extern "C" {

// Rebuilds the weight image from the BF16 weights (after every change of them),
// on the legacy default stream like the weight updates themselves.
static void refresh_weight_image(tg_mlp* m) {
  const int K1 = (m->NM + 15) / 16 * 16;
  const int n = m->H * K1 + m->H * m->H + 3 * m->H + 4;
  mlp_weight_image_kernel<<<(unsigned)((n + 255) / 256), 256>>>(m->d_wb, MlpLayout{m->NM, m->H}, K1,
                                                                m->d_wimg);
}

int tg_mlp_create(int32_t ndims, int32_t polydeg, int32_t hidden, uint64_t seed, tg_mlp** out) {
  if (!out) return mfail(nullptr, TG_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const int N = polydeg + 1;
  if ((ndims != 2 && ndims != 3) || N < 3 || N > 5)
    return mfail(nullptr, TG_ERR_UNSUPPORTED, "learned indicator: 2D/3D, polydeg 2..4");
  const int NM = ndims == 2 ? N * N : N * N * N;
  const int H = hidden > 0 ? hidden : (ndims == 2 ? 64 : 128);
  const bool ok = (NM == 16 && H == 64) || (NM == 9 && H == 64) || (NM == 25 && H == 64) ||
                  (NM == 27 && H == 128) || (NM == 64 && H == 128);
  if (!ok) return mfail(nullptr, TG_ERR_UNSUPPORTED, "network shape not compiled");
  tg_mlp* m = new tg_mlp();
  m->D = ndims;
  m->N = N;
  m->NM = NM;
  m->H = H;
  const MlpLayout L{NM, H};
  m->nparams = L.count();
  m->sqrt_threshold = std::sqrt(0.5 * std::pow(10.0, -1.8 * std::pow((double)N, 0.25)));
  // He-uniform initialisation from a fixed-seed LCG
  std::vector<float> w(m->nparams, 0.0f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return ((st >> 40) & 0xffffff) / 16777216.0f * 2.0f - 1.0f;
  };
  for (int i = 0; i < H * NM; ++i) w[L.w1() + i] = uni() * std::sqrt(6.0f / NM);
  for (int i = 0; i < H * H; ++i) w[L.w2() + i] = uni() * std::sqrt(6.0f / H);
  for (int i = 0; i < H; ++i) w[L.w3() + i] = uni() * std::sqrt(3.0f / H);
  w[L.b3()] = 0.0f;
  const size_t pb = sizeof(float) * m->nparams;
  cudaError_t e = cudaSuccess;
  e = e ? e : cudaMalloc(&m->d_w, pb);
  e = e ? e : cudaMalloc(&m->d_wb, sizeof(__nv_bfloat16) * m->nparams);
  {
    const int K1 = (NM + 15) / 16 * 16;
    m->wimg_bytes = (size_t)H * K1 * 2 + (size_t)H * H * 2 + (size_t)(3 * H + 4) * 4;
  }
  e = e ? e : cudaMalloc(&m->d_wimg, m->wimg_bytes);
  e = e ? e : cudaMalloc(&m->d_g, pb);
  e = e ? e : cudaMalloc(&m->d_m, pb);
  e = e ? e : cudaMalloc(&m->d_v, pb);
  e = e ? e : cudaMalloc(&m->d_loss, 2 * sizeof(float));
  e = e ? e : cudaMalloc(&m->d_stats, 3 * sizeof(unsigned long long));
  e = e ? e : cudaMalloc(&m->d_status, sizeof(int32_t));
  if (e != cudaSuccess) {
    delete m;
    return mfail(nullptr, TG_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaMemcpy(m->d_w, w.data(), pb, cudaMemcpyHostToDevice);
  cudaMemset(m->d_g, 0, pb);
  cudaMemset(m->d_m, 0, pb);
  cudaMemset(m->d_v, 0, pb);
  cudaMemset(m->d_stats, 0, 3 * sizeof(unsigned long long));
  to_bf16_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(m->d_w, m->d_wb, m->nparams);
  refresh_weight_image(m);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return mfail(nullptr, TG_ERR_CUDA, cudaGetErrorString(e));
  *out = m;
  return TG_OK;
}

int tg_mlp_destroy(tg_mlp* m) {
  if (!m) return TG_ERR_INVALID_ARGUMENT;
  void* ptrs[] = {m->d_w, m->d_wb, m->d_wimg, m->d_g, m->d_m, m->d_v, m->d_x, m->d_y, m->d_loss,
                  m->d_gpart, m->d_lpart,
                  m->d_pred, m->d_hg, m->d_flag, m->d_stats, m->d_status};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete m;
  return TG_OK;
}

int tg_mlp_nparams(const tg_mlp* m, int64_t* n) {
  if (!m || !n) return TG_ERR_INVALID_ARGUMENT;
  *n = m->nparams;
  return TG_OK;
}

int tg_mlp_get_params(tg_mlp* m, float* host) {
  if (!m || !host) return TG_ERR_INVALID_ARGUMENT;
  MCUDA(m, cudaMemcpy(host, m->d_w, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost));
  return TG_OK;
}

int tg_mlp_set_params(tg_mlp* m, const float* host) {
  if (!m || !host) return TG_ERR_INVALID_ARGUMENT;
  MCUDA(m, cudaMemcpy(m->d_w, host, sizeof(float) * m->nparams, cudaMemcpyHostToDevice));
  to_bf16_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(m->d_w, m->d_wb, m->nparams);
  refresh_weight_image(m);
  MCUDA(m, cudaDeviceSynchronize());
  return TG_OK;
}

// Appends the features/targets of every `stride`-th element of the context
// state (offset `phase`) to the training set (grown on demand).
int tg_mlp_harvest(tg_mlp* m, tg_ctx* c, int32_t stride, int32_t phase, int64_t* total) {
  if (!m || !c || stride < 1) return TG_ERR_INVALID_ARGUMENT;
  cudaStream_t s;
  int64_t E;
  // scratch for the full element set
  {
    const void* st;
    int ff, D, N;
    double g;
    const double* vi;
    void* strm;
    int rc = ctx_state_view(c, &st, &ff, &D, &N, &E, &g, &vi, &strm);
    if (rc) return rc;
  }
  float *feat = nullptr, *tgt = nullptr, *hg = nullptr;
  int32_t* flag = nullptr;
  MCUDA(m, cudaMalloc(&feat, sizeof(float) * E * m->NM));
  MCUDA(m, cudaMalloc(&tgt, sizeof(float) * E));
  MCUDA(m, cudaMalloc(&hg, sizeof(float) * E));
  MCUDA(m, cudaMalloc(&flag, sizeof(int32_t) * E));
  int rc = launch_features(m, c, feat, tgt, hg, flag, &s, &E);
  if (rc == TG_OK) {
    const int64_t take = (E - phase + stride - 1) / stride;
    if (m->count + take > m->cap) {
      const int64_t ncap = std::max<int64_t>(2 * m->cap, m->count + take);
      float *nx = nullptr, *ny = nullptr;
      cudaMalloc(&nx, sizeof(float) * ncap * m->NM);
      cudaMalloc(&ny, sizeof(float) * ncap);
      if (m->count) {
        cudaMemcpyAsync(nx, m->d_x, sizeof(float) * m->count * m->NM, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(ny, m->d_y, sizeof(float) * m->count, cudaMemcpyDeviceToDevice, s);
      }
      cudaStreamSynchronize(s);
      cudaFree(m->d_x);
      cudaFree(m->d_y);
      m->d_x = nx;
      m->d_y = ny;
      m->cap = ncap;
    }
    // strided gather of rows (pitched 2D copies)
    cudaMemcpy2DAsync(m->d_x + m->count * m->NM, sizeof(float) * m->NM, feat + phase * m->NM,
                      sizeof(float) * m->NM * stride, sizeof(float) * m->NM, take,
                      cudaMemcpyDeviceToDevice, s);
    cudaMemcpy2DAsync(m->d_y + m->count, sizeof(float), tgt + phase, sizeof(float) * stride,
                      sizeof(float), take, cudaMemcpyDeviceToDevice, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = mfail(m, TG_ERR_CUDA, cudaGetErrorString(e));
    else m->count += take;
  }
  cudaFree(feat);
  cudaFree(tgt);
  cudaFree(hg);
  cudaFree(flag);
  if (total) *total = m->count;
  return rc;
}

// Adam training on the harvested set: `steps` minibatches of `batch` samples
// drawn with replacement (rows i with i % holdout == 0 are held out when
// holdout > 1).  *mean_loss receives the mean squared error over all steps.
int tg_mlp_train(tg_mlp* m, int64_t steps, int32_t batch, float lr, int32_t holdout,
                 uint64_t seed, float* mean_loss) {
  if (!m || steps < 0 || batch < 1) return TG_ERR_INVALID_ARGUMENT;
  if (m->count < 2) return mfail(m, TG_ERR_STATE, "no training data harvested");
  MCUDA(m, cudaMemset(m->d_loss, 0, 2 * sizeof(float)));
  for (int64_t it = 0; it < steps; ++it) {
    const uint64_t sd = seed * 1000003ull + (uint64_t)(m->adam_t + 1);
    int rc = train_pass(m, m->d_x, m->d_y, m->count, nullptr, sd, batch, holdout);
    if (rc) return rc;
    m->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)m->adam_t), c2 = 1.0f - std::pow(b2, (float)m->adam_t);
    adam_kernel<<<(unsigned)((m->nparams + 255) / 256), 256>>>(m->d_w, m->d_wb, m->d_g, m->d_m,
                                                              m->d_v, m->nparams, lr, b1, b2, 1e-8f,
                                                              c1, c2);
  }
  if (steps > 0) refresh_weight_image(m);
  float l[2] = {0, 0};
  MCUDA(m, cudaMemcpy(l, m->d_loss, sizeof(l), cudaMemcpyDeviceToHost));
  if (mean_loss) *mean_loss = l[1] > 0 ? l[0] / l[1] : 0.0f;
  return TG_OK;
}

// Gradient of the mean squared error over explicit rows (x_host [n][NM],
// y_host [n]) at the current weights, written to grad_host [nparams] (FP32),
// without changing the weights: the check against the CPU oracle.
int tg_mlp_gradient(tg_mlp* m, const float* x_host, const float* y_host, int32_t n,
                    float* grad_host, float* loss_host) {
  if (!m || !x_host || !y_host || !grad_host || n < 1) return TG_ERR_INVALID_ARGUMENT;
  float *x = nullptr, *y = nullptr;
  int64_t* idx = nullptr;
  MCUDA(m, cudaMalloc(&x, sizeof(float) * n * m->NM));
  MCUDA(m, cudaMalloc(&y, sizeof(float) * n));
  MCUDA(m, cudaMalloc(&idx, sizeof(int64_t) * n));
  std::vector<int64_t> id(n);
  for (int i = 0; i < n; ++i) id[i] = i;
  cudaMemcpy(x, x_host, sizeof(float) * n * m->NM, cudaMemcpyHostToDevice);
  cudaMemcpy(y, y_host, sizeof(float) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(idx, id.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice);
  cudaMemset(m->d_loss, 0, 2 * sizeof(float));
  const int rc = train_pass(m, x, y, n, idx, 0, n, 0);
  if (rc) {
    cudaFree(x);
    cudaFree(y);
    cudaFree(idx);
    return rc;
  }
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(grad_host, m->d_g, sizeof(float) * m->nparams, cudaMemcpyDeviceToHost);
  float l[2];
  if (e == cudaSuccess) e = cudaMemcpy(l, m->d_loss, sizeof(l), cudaMemcpyDeviceToHost);
  if (loss_host && e == cudaSuccess) *loss_host = l[0] / n;
  cudaMemset(m->d_g, 0, sizeof(float) * m->nparams);
  cudaFree(x);
  cudaFree(y);
  cudaFree(idx);
  if (e != cudaSuccess) return mfail(m, TG_ERR_CUDA, cudaGetErrorString(e));
  return TG_OK;
}

// Network predictions (sqrt E) for explicit rows x_host [n][NM], by the same
// tensor-core kernel as the deployment.
int tg_mlp_predict(tg_mlp* m, const float* x_host, int64_t n, float* pred_host) {
  if (!m || !x_host || !pred_host || n < 1) return TG_ERR_INVALID_ARGUMENT;
  float *x = nullptr, *p = nullptr;
  MCUDA(m, cudaMalloc(&x, sizeof(float) * n * m->NM));
  cudaError_t e = cudaMalloc(&p, sizeof(float) * n);
  if (e == cudaSuccess) e = cudaMemcpy(x, x_host, sizeof(float) * n * m->NM, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_status, 0, sizeof(int32_t));
  int rc = e == cudaSuccess ? launch_predict(m, x, n, p, 0) : TG_OK;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int32_t st = 0;
  if (rc == TG_OK && e == cudaSuccess) e = cudaMemcpy(&st, m->d_status, sizeof(st), cudaMemcpyDeviceToHost);
  if (rc == TG_OK && e == cudaSuccess) e = cudaMemcpy(pred_host, p, sizeof(float) * n, cudaMemcpyDeviceToHost);
  cudaFree(x);
  cudaFree(p);
  if (rc) return rc;
  if (e != cudaSuccess) return mfail(m, TG_ERR_CUDA, cudaGetErrorString(e));
  if (st) return mfail(m, TG_ERR_CUDA, "tensor-core MLP: a wait for the tensor core timed out");
  return TG_OK;
}

// Harvested rows (features, targets) copied to the host (count from tg_mlp_harvest).
int tg_mlp_dataset(tg_mlp* m, float* x_host, float* y_host) {
  if (!m || !x_host || !y_host) return TG_ERR_INVALID_ARGUMENT;
  MCUDA(m, cudaMemcpy(x_host, m->d_x, sizeof(float) * m->count * m->NM, cudaMemcpyDeviceToHost));
  MCUDA(m, cudaMemcpy(y_host, m->d_y, sizeof(float) * m->count, cudaMemcpyDeviceToHost));
  return TG_OK;
}

// Use the network as the context's shock indicator (band: half-width of the
// fallback zone in sqrt(E) around sqrt of the HG threshold).  m == NULL
// restores the Hennemann-Gassner indicator.
int tg_ctx_set_learned_indicator(tg_ctx* c, tg_mlp* m, float band) {
  if (!c) return TG_ERR_INVALID_ARGUMENT;
  if (m) {
    const void* st;
    int ff, D, N;
    int64_t E;
    double g;
    const double* vi;
    void* strm;
    int rc = ctx_state_view(c, &st, &ff, &D, &N, &E, &g, &vi, &strm);
    if (rc) return rc;
    if (D != m->D || N != m->N) return mfail(m, TG_ERR_INVALID_ARGUMENT, "network/context shape mismatch");
    if (E > m->ecap) {
      cudaFree(m->d_pred);
      cudaFree(m->d_hg);
      cudaFree(m->d_flag);
      MCUDA(m, cudaMalloc(&m->d_pred, sizeof(float) * E));
      MCUDA(m, cudaMalloc(&m->d_hg, sizeof(float) * E));
      MCUDA(m, cudaMalloc(&m->d_flag, sizeof(int32_t) * E));
      m->ecap = E;
    }
    m->band = band;
  }
  return ctx_set_alpha_source(c, m);
}

// Learned-indicator diagnostics of the last stage: per element the network's
// blending factor inputs (pred: predicted sqrt E), the HG factor (hg, with
// alpha_min = 0 and alpha_max = 1) and the fallback flag, plus the running
// counts {elements evaluated, band fallbacks, positivity fallbacks}.
int tg_mlp_last(tg_mlp* m, float* pred, float* hg, int32_t* flag, uint64_t* counts) {
  if (!m) return TG_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  if (pred) MCUDA(m, cudaMemcpy(pred, m->d_pred, sizeof(float) * m->ecap, cudaMemcpyDeviceToHost));
  if (hg) MCUDA(m, cudaMemcpy(hg, m->d_hg, sizeof(float) * m->ecap, cudaMemcpyDeviceToHost));
  if (flag) MCUDA(m, cudaMemcpy(flag, m->d_flag, sizeof(int32_t) * m->ecap, cudaMemcpyDeviceToHost));
  if (counts) MCUDA(m, cudaMemcpy(counts, m->d_stats, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  return TG_OK;
}

}  // extern "C"
