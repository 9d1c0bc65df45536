/*
 * Calls libtrixi_gb300 the way the Julia drop-in (trixi.jl_gb300/julia/TrixiGB300.jl)
 * does, from plain C with no CUDA of its own: a tg_config pointing at Trixi's
 * own arrays (1-based Int64 neighbor_ids [2, ninterfaces] and column-major basis
 * matrices, as in cache.interfaces and dg.basis), the state in device vectors
 * owned by the library (the shim's GB300Array: OrdinaryDiffEq's u, du and tmp),
 * rhs_hyperbolic! through tg_rhs on those vectors, and CarpenterKennedy2N54 in
 * OrdinaryDiffEq's broadcast form (tmp = A tmp + dt du; u = u + B tmp) through
 * tg_lincomb, with a fixed step.  Test driver for tests/test_gpu_shim_abi.py.
 *
 *   shim_driver <input> <output>
 *
 * Input (little-endian, written by the test): int64 ndims, polydeg, nelements,
 * ninterfaces, volume_integral, volume_flux, surface_flux, volume_flux_fv,
 * alpha_smooth, source_terms, precision, nsteps; double gamma, alpha_max,
 * alpha_min, t0, dt; double A[5], B[5], c[5]; double nodes[n], weights[n],
 * inverse_weights[n], derivative_hat[n n], derivative_split[n n],
 * inverse_vandermonde_legendre[n n]; int64 neighbor_ids[2 I], orientations[I];
 * double inverse_jacobian[E], node_coordinates[ndims n^ndims E],
 * u0[nvars n^ndims E].
 * Output: double du0[nvalues] (rhs at t0), u_end[nvalues] (after nsteps),
 * max_dt (of u_end).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "trixi_gb300.h"

static FILE* in_file;

static void die(const char* what, tg_ctx* ctx) {
  char buf[512];
  tg_last_error(ctx, buf, sizeof(buf));
  fprintf(stderr, "shim_driver: %s: %s\n", what, buf);
  exit(1);
}

static void* read_array(size_t count, size_t size) {
  void* p = malloc(count * size + 1);
  if (!p || fread(p, size, count, in_file) != count) {
    fprintf(stderr, "shim_driver: short input\n");
    exit(1);
  }
  return p;
}

#define CHECK(call, ctx, what) \
  do {                         \
    if ((call) != TG_OK) die(what, ctx); \
  } while (0)

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: shim_driver <input> <output>\n");
    return 2;
  }
  in_file = fopen(argv[1], "rb");
  if (!in_file) {
    perror(argv[1]);
    return 1;
  }
  int64_t* h = (int64_t*)read_array(12, sizeof(int64_t));
  double* hd = (double*)read_array(5, sizeof(double));
  double* A = (double*)read_array(5, sizeof(double));
  double* B = (double*)read_array(5, sizeof(double));
  double* C = (double*)read_array(5, sizeof(double));
  const int64_t ndims = h[0], polydeg = h[1], E = h[2], I = h[3], nsteps = h[11];
  const int64_t n = polydeg + 1;
  int64_t nn = 1;
  for (int d = 0; d < ndims; ++d) nn *= n;
  const int64_t nvalues = (ndims + 2) * nn * E;

  tg_config cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.ndims = (int32_t)ndims;
  cfg.polydeg = (int32_t)polydeg;
  cfg.nelements = E;
  cfg.ninterfaces = I;
  cfg.volume_integral = (int32_t)h[4];
  cfg.volume_flux = (int32_t)h[5];
  cfg.surface_flux = (int32_t)h[6];
  cfg.volume_flux_fv = (int32_t)h[7];
  cfg.alpha_smooth = (int32_t)h[8];
  cfg.source_terms = (int32_t)h[9];
  cfg.precision = (int32_t)h[10];
  cfg.gamma = hd[0];
  cfg.alpha_max = hd[1];
  cfg.alpha_min = hd[2];
  cfg.nodes = (const double*)read_array(n, sizeof(double));
  cfg.weights = (const double*)read_array(n, sizeof(double));
  cfg.inverse_weights = (const double*)read_array(n, sizeof(double));
  cfg.derivative_hat = (const double*)read_array(n * n, sizeof(double));
  cfg.derivative_split = (const double*)read_array(n * n, sizeof(double));
  cfg.inverse_vandermonde_legendre = (const double*)read_array(n * n, sizeof(double));
  cfg.neighbor_ids = (const int64_t*)read_array(2 * I, sizeof(int64_t));
  cfg.orientations = (const int64_t*)read_array(I, sizeof(int64_t));
  cfg.inverse_jacobian = (const double*)read_array(E, sizeof(double));
  cfg.node_coordinates = (const double*)read_array(ndims * nn * E, sizeof(double));
  double* u0 = (double*)read_array(nvalues, sizeof(double));
  fclose(in_file);

  tg_ctx* ctx = NULL;
  CHECK(tg_ctx_create(&cfg, &ctx), NULL, "tg_ctx_create");

  /* the integrator's vectors, in device memory the library owns */
  double *u, *du, *tmp;
  CHECK(tg_vector_create(ctx, nvalues, &u), ctx, "tg_vector_create");
  CHECK(tg_vector_create(ctx, nvalues, &du), ctx, "tg_vector_create");
  CHECK(tg_vector_create(ctx, nvalues, &tmp), ctx, "tg_vector_create");
  CHECK(tg_vector_copy(ctx, u, u0, nvalues, 0), ctx, "upload");

  double* out = (double*)malloc(sizeof(double) * (2 * nvalues + 1));
  const double t0 = hd[3], dt = hd[4];
  CHECK(tg_rhs(ctx, du, u, t0), ctx, "tg_rhs");
  CHECK(tg_vector_copy(ctx, out, du, nvalues, 1), ctx, "download du");

  /* CarpenterKennedy2N54 as OrdinaryDiffEq broadcasts it, fixed dt */
  double t = t0;
  for (int64_t step = 0; step < nsteps; ++step) {
    for (int s = 0; s < 5; ++s) {
      CHECK(tg_rhs(ctx, du, u, t + C[s] * dt), ctx, "tg_rhs");
      if (s == 0)
        CHECK(tg_lincomb(ctx, nvalues, tmp, dt, du, 0.0, NULL), ctx, "tg_lincomb");
      else
        CHECK(tg_lincomb(ctx, nvalues, tmp, A[s], tmp, dt, du), ctx, "tg_lincomb");
      CHECK(tg_lincomb(ctx, nvalues, u, 1.0, u, B[s], tmp), ctx, "tg_lincomb");
    }
    t += dt;
  }
  CHECK(tg_vector_copy(ctx, out + nvalues, u, nvalues, 1), ctx, "download u");
  CHECK(tg_max_dt(ctx, u, out + 2 * nvalues), ctx, "tg_max_dt");

  CHECK(tg_vector_destroy(ctx, tmp), ctx, "tg_vector_destroy");
  CHECK(tg_ctx_destroy(ctx), ctx, "tg_ctx_destroy");  /* frees u and du too */
  FILE* f = fopen(argv[2], "wb");
  if (!f || fwrite(out, sizeof(double), 2 * nvalues + 1, f) != (size_t)(2 * nvalues + 1)) {
    fprintf(stderr, "shim_driver: cannot write %s\n", argv[2]);
    return 1;
  }
  fclose(f);
  return 0;
}
