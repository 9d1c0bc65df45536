// Domain integrals of a state without any device allocation.
//
// tg_integrals() needs a context, and creating one allocates device memory.
// Some callers cannot allocate: code running inside a memory pool that must
// not grow, a host that captures work into a CUDA graph while allocations are
// forbidden, or a runtime that owns all device memory itself and hands out
// only the buffers it manages (a Julia GPU array, a pre-sized arena).  For
// them, tg_integrals_noalloc() evaluates the same FP64 integrals from
// caller-owned input and output buffers, using as scratch a fixed array in
// the library's static device memory instead of cudaMalloc.
//
// The scratch holds one partial sum per chunk of TG_NOALLOC_CHUNK elements,
// so the largest mesh is TG_NOALLOC_MAX_CHUNKS * TG_NOALLOC_CHUNK elements;
// every GPU that loads the library keeps this 4 MiB array until the process
// exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/trixi_gb300.h"

namespace tg {
// Message for tg_last_error(NULL, ...) of the calling thread (tg_api.cu).
void set_thread_error(const char* msg);
}  // namespace tg

#define TG_NOALLOC_CHUNK 64
#define TG_NOALLOC_MAX_CHUNKS 65536
#define TG_NOALLOC_K 8  // per-chunk slots: up to 5 conserved totals, entropy, kinetic energy

// Shared by every call on a device; each call overwrites the chunks it uses
// before reading them, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_noalloc_partials[TG_NOALLOC_MAX_CHUNKS * TG_NOALLOC_K];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch[kMaxDevices] = {nullptr};
void* g_scratch_ctx[kMaxDevices] = {nullptr};  // the context each address was resolved in

// The calling thread's current driver context (CUcontext), through the
// runtime's driver entry point so that the library needs no link to libcuda;
// nullptr when it cannot be queried or no context is current yet.
void* current_context() {
  using Fn = int (*)(void**);
  static Fn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (Fn)p;
  }();
  void* ctx = nullptr;
  if (fn && fn(&ctx) != 0) ctx = nullptr;
  return ctx;
}

struct NoallocParams {
  int D, N, NV;
  int64_t E;
  double gamma;
  double weights[8];
};

// One element per thread; each block reduces its TG_NOALLOC_CHUNK elements in
// a fixed order into one partial (integrate_via_indices, analysis_dg2d.jl:313-336).
__global__ void noalloc_chunk_kernel(NoallocParams P, const double* __restrict__ u,
                                     const double* __restrict__ inv_jac,
                                     double* __restrict__ partials) {
  __shared__ double sh[TG_NOALLOC_CHUNK][TG_NOALLOC_K];
  const int tid = threadIdx.x;
  const int64_t e = (int64_t)blockIdx.x * TG_NOALLOC_CHUNK + tid;
  const int NV = P.NV, N = P.N, D = P.D;
  const int K = NV + 2;
  double acc[TG_NOALLOC_K];
  for (int k = 0; k < TG_NOALLOC_K; ++k) acc[k] = 0.0;
  if (e < P.E) {
    const int NN = D == 2 ? N * N : N * N * N;
    double vj = 1.0 / inv_jac[e];
    vj = D == 2 ? vj * vj : vj * vj * vj;
    for (int q = 0; q < NN; ++q) {
      const int i = q % N, j = (q / N) % N, kk = q / (N * N);
      double w = P.weights[i] * P.weights[j];
      if (D == 3) w *= P.weights[kk];
      const double* p = u + ((size_t)e * NN + q) * NV;
      double m2 = 0;
      for (int d = 0; d < D; ++d) m2 += p[1 + d] * p[1 + d];
      for (int v = 0; v < NV; ++v) acc[v] += vj * w * p[v];
      const double pr = (P.gamma - 1) * (p[NV - 1] - 0.5 * m2 / p[0]);
      const double s = log(pr) - P.gamma * log(p[0]);
      acc[NV] += vj * w * (-s * p[0] / (P.gamma - 1));
      acc[NV + 1] += vj * w * (m2 / (2 * p[0]));
    }
  }
  for (int k = 0; k < K; ++k) sh[tid][k] = acc[k];
  __syncthreads();
  for (int w = TG_NOALLOC_CHUNK / 2; w > 0; w >>= 1) {
    if (tid < w)
      for (int k = 0; k < K; ++k) sh[tid][k] += sh[tid + w][k];
    __syncthreads();
  }
  if (tid < K) partials[(size_t)blockIdx.x * TG_NOALLOC_K + tid] = sh[0][tid];
}

// Sum of the chunk partials in a fixed order (one block).
__global__ void noalloc_sum_kernel(const double* __restrict__ partials, int64_t nchunks, int K,
                                   double* __restrict__ out) {
  __shared__ double sh[256];
  for (int k = 0; k < K; ++k) {
    double s = 0;
    for (int64_t c = threadIdx.x; c < nchunks; c += blockDim.x) s += partials[c * TG_NOALLOC_K + k];
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

int fail(int code, const char* msg) {
  tg::set_thread_error(msg);
  return code;
}

}  // namespace

extern "C" int tg_integrals_noalloc(int32_t ndims, int32_t polydeg, int64_t nelements, double gamma,
                                    const double* weights, const double* u_dev,
                                    const double* inverse_jacobian_dev, double* out_dev,
                                    void* stream) {
  if (ndims != 2 && ndims != 3) return fail(TG_ERR_INVALID_ARGUMENT, "ndims must be 2 or 3");
  if (polydeg < 1 || polydeg > 7) return fail(TG_ERR_INVALID_ARGUMENT, "polydeg must be 1..7");
  if (!weights || !u_dev || !inverse_jacobian_dev || !out_dev)
    return fail(TG_ERR_INVALID_ARGUMENT, "null argument");
  if (nelements <= 0) return fail(TG_ERR_INVALID_ARGUMENT, "nelements must be > 0");
  const int64_t nchunks = (nelements + TG_NOALLOC_CHUNK - 1) / TG_NOALLOC_CHUNK;
  if (nchunks > TG_NOALLOC_MAX_CHUNKS) {
    char buf[160];
    snprintf(buf, sizeof(buf),
             "tg_integrals_noalloc: %lld elements exceed the static scratch limit of %d",
             (long long)nelements, TG_NOALLOC_MAX_CHUNKS * TG_NOALLOC_CHUNK);
    return fail(TG_ERR_INVALID_ARGUMENT, buf);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(TG_ERR_CUDA, "tg_integrals_noalloc: no current CUDA device");
  double* scratch;
  {
    // First call on this device (or in a context other than the one the
    // address was resolved in, e.g. after cudaDeviceReset or under a
    // non-primary context): resolve the device address of the static scratch
    // array (its host-side name is only a stand-in).
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev] || g_scratch_ctx[dev] != current_context()) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_partials);
      if (e != cudaSuccess || !p)
        return fail(TG_ERR_CUDA, "tg_integrals_noalloc: cudaGetSymbolAddress failed");
      g_scratch[dev] = (double*)p;
      g_scratch_ctx[dev] = current_context();  // current now: the call above set it up
    }
    scratch = g_scratch[dev];
  }
  NoallocParams P{};
  P.D = ndims;
  P.N = polydeg + 1;
  P.NV = ndims + 2;
  P.E = nelements;
  P.gamma = gamma;
  for (int i = 0; i < P.N; ++i) P.weights[i] = weights[i];
  cudaStream_t s = (cudaStream_t)stream;
  noalloc_chunk_kernel<<<(unsigned)nchunks, TG_NOALLOC_CHUNK, 0, s>>>(P, u_dev, inverse_jacobian_dev,
                                                                      scratch);
  noalloc_sum_kernel<<<1, 256, 0, s>>>(scratch, nchunks, P.NV + 2, out_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(TG_ERR_CUDA, cudaGetErrorString(e));
  return TG_OK;
}

