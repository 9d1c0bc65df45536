// Explicit instantiation of the FP64 element kernels for one (dimension,
// volume integral) pair.  Each tg_inst_*.cu unit defines TG_D,
// TG_REAL and TG_VI and includes this file, so the instantiations compile in
// parallel.
#include "tg_dg.cuh"

#ifndef TG_D
#error "TG_D must be defined"
#endif

namespace tg {

template <int D, int N, typename R, int VI, int EPB>
static int launch_one(const DgParams& P, const StageArgs& A, cudaStream_t s) {
  using K = ElementKernel<D, N, R, R, VI, EPB>;
  auto kern = dg_element_kernel<D, N, R, R, VI, EPB>;
  static bool configured = false;
  const size_t smem = K::smem_bytes();
  if (!configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return -1;
    configured = true;
  }
  const int64_t nblocks = (P.nelements + EPB - 1) / EPB;
  if (nblocks <= 0) return 0;
  kern<<<(unsigned)nblocks, K::NT, smem, s>>>(P, A);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

#define TG_CAT2(a, b) a##b
#define TG_CAT(a, b) TG_CAT2(a, b)

// Elements-per-block choices compiled for each N (the first is the default).
// 2D: 256 threads per block by default; 3D likewise (N^3 nodes per element).
int TG_CAT(launch_element_, TG_SUFFIX)(int N, int epb, const DgParams& P, const StageArgs& A,
                                       cudaStream_t s) {
#if TG_D == 2
  switch (N) {
    case 2: return launch_one<2, 2, TG_REAL, TG_VI, 64>(P, A, s);
    case 3: return launch_one<2, 3, TG_REAL, TG_VI, 28>(P, A, s);
    case 4:
      if (epb == 8) return launch_one<2, 4, TG_REAL, TG_VI, 8>(P, A, s);
      if (epb == 32) return launch_one<2, 4, TG_REAL, TG_VI, 32>(P, A, s);
      return launch_one<2, 4, TG_REAL, TG_VI, 16>(P, A, s);
    case 5: return launch_one<2, 5, TG_REAL, TG_VI, 10>(P, A, s);
    case 6: return launch_one<2, 6, TG_REAL, TG_VI, 7>(P, A, s);
  }
#else
  switch (N) {
    case 2: return launch_one<3, 2, TG_REAL, TG_VI, 32>(P, A, s);
    case 3: return launch_one<3, 3, TG_REAL, TG_VI, 9>(P, A, s);
    case 4:
      if (epb == 2) return launch_one<3, 4, TG_REAL, TG_VI, 2>(P, A, s);
      if (epb == 8) return launch_one<3, 4, TG_REAL, TG_VI, 8>(P, A, s);
      return launch_one<3, 4, TG_REAL, TG_VI, 4>(P, A, s);
    case 5: return launch_one<3, 5, TG_REAL, TG_VI, 2>(P, A, s);
  }
#endif
  return -2;
}

#if TG_VI == 2
template <int D, int N, typename R, int EPB>
static int launch_ind(const DgParams& P, const double* u, void* alpha, cudaStream_t s) {
  const int64_t nblocks = (P.nelements + EPB - 1) / EPB;
  if (nblocks <= 0) return 0;
  hg_indicator_kernel<D, N, R, EPB, DgParams, double>
      <<<(unsigned)nblocks, EPB * Pow<N, D>::value, 0, s>>>(P, u, reinterpret_cast<R*>(alpha));
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int TG_CAT(launch_indicator_, TG_SUFFIX)(int N, const DgParams& P, const double* u, void* alpha,
                                         cudaStream_t s) {
#if TG_D == 2
  switch (N) {
    case 2: return launch_ind<2, 2, TG_REAL, 64>(P, u, alpha, s);
    case 3: return launch_ind<2, 3, TG_REAL, 28>(P, u, alpha, s);
    case 4: return launch_ind<2, 4, TG_REAL, 16>(P, u, alpha, s);
    case 5: return launch_ind<2, 5, TG_REAL, 10>(P, u, alpha, s);
    case 6: return launch_ind<2, 6, TG_REAL, 7>(P, u, alpha, s);
  }
#else
  switch (N) {
    case 2: return launch_ind<3, 2, TG_REAL, 32>(P, u, alpha, s);
    case 3: return launch_ind<3, 3, TG_REAL, 9>(P, u, alpha, s);
    case 4: return launch_ind<3, 4, TG_REAL, 4>(P, u, alpha, s);
    case 5: return launch_ind<3, 5, TG_REAL, 2>(P, u, alpha, s);
  }
#endif
  return -2;
}
#endif

}  // namespace tg
