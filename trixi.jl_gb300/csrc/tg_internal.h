// Interfaces between the library's translation units (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "../../include/trixi_gb300.h"
#include "tg_mixed.cuh"

namespace tg {

// What the ensemble (tg_ensemble.cu) needs of one context.
struct CtxView {
  const MixedParams* mp;  // host copy of the mixed-precision parameters
  void* u[2];             // state buffers (float-float in mixed contexts)
  int cur;                // which of them holds the state
  void* utmp;             // 2N register
  Clock* clock;           // device clock
  int32_t* status;        // sticky device status word
  int D, N, vi, fp64, epb;
  int64_t E;
  cudaStream_t stream;
  bool uploaded;
};

int ctx_view(tg_ctx* c, CtxView* v);
void ctx_set_cur(tg_ctx* c, int cur);
// initialize!(StepsizeCallback) on the first call (dt = cfl * max_dt(u) at
// t0), otherwise a new t_end and cfl, on the context's stream; with `sync`
// it returns after the clock is set.
int ctx_clock_prepare(tg_ctx* c, double t0, double t_end, double cfl, bool sync);
// message for tg_last_error(NULL, ...) of the calling thread
void set_thread_error(const char* msg);

}  // namespace tg
