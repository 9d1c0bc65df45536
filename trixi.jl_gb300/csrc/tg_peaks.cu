// FMA issue-rate microbenchmark of the current device (FP32 or FP64): the
// compute-side denominator the element kernels' arithmetic rate is compared
// with.  Every thread runs 8 independent FMA chains; a full-occupancy grid of
// 8 blocks x 256 threads per SM keeps every FMA pipe busy.  Timed with CUDA
// events on a private stream after a warm-up launch.
#include <cuda_runtime.h>

#include "../../include/trixi_gb300.h"

namespace tg {
void set_thread_error(const char* msg);
}

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + 1) * (T)1e-3 + (T)k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == (T)-1) out[0] = s;  // never true: keeps the chains alive
}

template <typename T>
int run(int iters, double* flops_per_second) {
  int dev = 0, sms = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  T* out = nullptr;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMalloc(&out, sizeof(T));
  const unsigned blocks = (unsigned)sms * 8;
  float ms = 0;
  if (e == cudaSuccess) {
    fma_chain_kernel<T><<<blocks, 256, 0, st>>>(out, iters, (T)0.999999, (T)1e-6);  // warm-up
    cudaEventRecord(e0, st);
    fma_chain_kernel<T><<<blocks, 256, 0, st>>>(out, iters, (T)0.999999, (T)1e-6);
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
  }
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (out) cudaFree(out);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) {
    tg::set_thread_error(cudaGetErrorString(e));
    return TG_ERR_CUDA;
  }
  *flops_per_second = 2.0 * 8.0 * (double)iters * blocks * 256.0 / (ms * 1e-3);
  return TG_OK;
}

}  // namespace

extern "C" int tg_fma_peak(int32_t fp64, double* flops_per_second) {
  if (!flops_per_second) return TG_ERR_INVALID_ARGUMENT;
  // about 20 GFLOP in FP32 and 2.5 GFLOP in FP64 (a few ms at the nominal rates)
  return fp64 ? run<double>(512, flops_per_second) : run<float>(4096, flops_per_second);
}
