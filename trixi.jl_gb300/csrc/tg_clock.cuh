// Device-side time-stepping clock shared by the single-context step graphs
// (tg_api.cu) and the ensemble (tg_ensemble.cu): the prologue and epilogue of
// SimpleIntegrator2N's step! with StepsizeCallback, on one Clock.
#pragma once

#include "tg_dg.cuh"

namespace tg {

// Host copies of the CarpenterKennedy2N54 coefficients (methods_2N.jl:24-48)
static const double CK_A[5] = {0.0, 567301805773.0 / 1357537059087.0,
                                2404267990393.0 / 2016746695238.0,
                                3550918686646.0 / 2091501179385.0,
                                1275806237668.0 / 842570457699.0};
static const double CK_B[5] = {1432997174477.0 / 9575080441755.0,
                               5161836677717.0 / 13612068292357.0,
                               1720146321549.0 / 2090206949498.0,
                               3134564353537.0 / 4481467310338.0,
                               2277821191437.0 / 14882151754819.0};
static const double CK_C[5] = {0.0, 1432997174477.0 / 9575080441755.0,
                               2526269341429.0 / 6820363962896.0,
                               2006345519317.0 / 3224310063776.0,
                               2802321613138.0 / 2924317926251.0};

// CarpenterKennedy2N54 stage times c_s (methods_2N.jl:39-44)
static __device__ const double CK_C_DEV[5] = {0.0, 1432997174477.0 / 9575080441755.0,
                                              2526269341429.0 / 6820363962896.0,
                                              2006345519317.0 / 3224310063776.0,
                                              2802321613138.0 / 2924317926251.0};

// sin/cos(pi t_s) of stage s as float-float pairs, for the mixed kernels'
// source phase
static __device__ __forceinline__ void stage_phase(Clock* c, int s) {
  double sn, cs;
  sincospi(c->t + CK_C_DEV[s] * c->dt, &sn, &cs);
  c->sin_t[s] = (float)sn;
  c->cos_t[s] = (float)cs;
  c->sin_tl[s] = (float)(sn - (double)c->sin_t[s]);
  c->cos_tl[s] = (float)(cs - (double)c->cos_t[s]);
}

static __device__ __forceinline__ void stage_phases(Clock* c) {
  for (int s = 0; s < 5; ++s) stage_phase(c, s);
}

// step! prologue: NaN check and limit_dt! (methods_2N.jl:131-140,
// time_integration.jl:46-55) and reset of the CFL reduction by lane 0 of a
// warp, then the five stage phases by lanes 0..4 (FP64 sincospi in parallel).
static __device__ __forceinline__ void clock_begin_warp(Clock* c) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    c->speed_bits = 1ull;  // nextfloat(0.0), where max_dt starts (stepsize_dg2d.jl:12)
    if (c->finished) {
      c->skip = 1;
    } else if (isnan(c->dt)) {
      c->nan_dt = 1;
      c->finished = 1;
      c->skip = 1;
    } else {
      c->skip = 0;
      const double tn = c->t + c->dt;
      const double te = c->t_end;
      // Julia isapprox: exact equality, or finite operands within rtol = sqrt(eps)
      const bool approx = tn == te || (isfinite(tn) && isfinite(te) &&
                                       fabs(tn - te) <= 1.4901161193847656e-08 * fmax(fabs(tn), fabs(te)));
      if (tn > te || approx) {
        c->dt = te - c->t;
        c->finalstep = 1;
      }
    }
  }
  __syncwarp();
  if (lane < 5 && !c->skip) stage_phase(c, lane);
}

// step! epilogue: t += dt, then StepsizeCallback: dt = cfl * max_dt(u_new)
// (stepsize.jl:93-126, max_dt = 2 / (nnodes * max scaled speed)).
static __device__ __forceinline__ void clock_end(Clock* c, int n) {
  if (c->skip) return;
  c->t += c->dt;
  c->steps += 1;
  const double speed = __longlong_as_double((long long)c->speed_bits);
  c->dt = c->cfl * (2.0 / (n * speed));
  if (c->finalstep) c->finished = 1;
}

}  // namespace tg
