/*
 * trixi_gb300.h -- C ABI of the GB300 (sm_103a) DGSEM hot path.
 *
 * Drop-in device backend for Trixi.jl's DGSEM semidiscretization of the
 * compressible Euler equations (2D/3D; TreeMesh periodic or not, with L2
 * mortars and AMR; curvilinear StructuredMesh / P4estMesh bricks).  The entry
 * points replace, one for one, the pieces of the reference that a Julia
 * `ccall` shim hands to the device (paths relative to the Trixi.jl sources):
 *
 *   rhs_hyperbolic!(du_ode, u_ode, semi, t)
 *       src/semidiscretization/semidiscretization_hyperbolic.jl:578-597
 *       -> dispatch rhs_hyperbolic!(backend, du, u, t, mesh::TreeMesh, ...)
 *          src/solvers/dgsem_tree/dg_2d.jl:113-186 (3D shares it, dg_2d.jl:117)
 *   the 2N low-storage Runge-Kutta stage and step
 *       src/time_integration/methods_2N.jl:131-168, time_integration.jl:46-55
 *   max_dt / StepsizeCallback
 *       src/callbacks_step/stepsize_dg2d.jl:8-30, stepsize_dg3d.jl:8-33,
 *       src/callbacks_step/stepsize.jl:93-126
 *   integrate_via_indices (conserved totals, entropy, kinetic energy)
 *       src/callbacks_step/analysis_dg2d.jl:313-336
 *   IndicatorHennemannGassner blending factors
 *       src/solvers/dgsem/indicators.jl:114-148,
 *       src/solvers/dgsem_tree/indicators_2d.jl:30-136, indicators_3d.jl:39-176
 *
 * Conventions
 *   - Every function returns an int status (TG_OK = 0, negative on error).  No
 *     exception, abort or device trap crosses the ABI; tg_last_error() gives
 *     the message of the last failure.
 *   - State arrays use Trixi's own layout u[v, i, j, (k), element]
 *     (column-major, variables fastest), FP64, ndofs * nvariables values.
 *   - The library owns the device memory of a context.  Host pointers are
 *     borrowed for the duration of a call; device pointers handed out stay
 *     valid until tg_ctx_destroy (the state pointer until the next tg_step or
 *     tg_rk_stage, see tg_state_device_ptr).
 *   - Calls are ordered on the context's CUDA stream.  One context per host
 *     thread; distinct contexts are independent.
 */
#ifndef TRIXI_GB300_H
#define TRIXI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_API_VERSION 3

typedef enum tg_status_code {
  TG_OK = 0,
  TG_ERR_INVALID_ARGUMENT = -1,
  TG_ERR_UNSUPPORTED = -2,   /* mesh/solver option outside the GPU path */
  TG_ERR_CUDA = -3,          /* a CUDA runtime call failed */
  TG_ERR_NUMERICAL = -4,     /* NaN time step or non-physical state detected */
  TG_ERR_STATE = -5          /* call order violated (e.g. no state uploaded) */
} tg_status_code;

/* VolumeIntegralWeakForm / VolumeIntegralFluxDifferencing /
 * VolumeIntegralShockCapturingHG, src/solvers/dg.jl:105, 135-141, 208-221 */
typedef enum tg_volume_integral {
  TG_VOLUME_WEAK_FORM = 0,
  TG_VOLUME_FLUX_DIFFERENCING = 1,
  TG_VOLUME_SHOCK_CAPTURING_HG = 2
} tg_volume_integral;

/* two-point fluxes: flux_central (numerical_fluxes.jl:17-25), flux_ranocha
 * (compressible_euler_2d.jl:686-722), flux_shima_etal (:466-495),
 * FluxLaxFriedrichs(max_abs_speed) = flux_lax_friedrichs and
 * FluxLaxFriedrichs(max_abs_speed_naive) (numerical_fluxes.jl:222-253),
 * flux_hllc (compressible_euler_2d.jl:1720-1816), flux_chandrashekar
 * (compressible_euler_2d.jl, 3d.jl:640-692), flux_hlle = FluxHLL(
 * min_max_speed_einfeldt) (numerical_fluxes.jl:422-457; HLLC and HLLE are
 * surface and FV subcell fluxes only, not flux-differencing volume fluxes) */
typedef enum tg_flux {
  TG_FLUX_CENTRAL = 0,
  TG_FLUX_RANOCHA = 1,
  TG_FLUX_SHIMA_ETAL = 2,
  TG_FLUX_LAX_FRIEDRICHS = 3,
  TG_FLUX_LAX_FRIEDRICHS_NAIVE = 4,
  TG_FLUX_HLLC = 5,
  TG_FLUX_CHANDRASHEKAR = 6,
  TG_FLUX_HLLE = 7
} tg_flux;

/* source_terms_convergence_test, compressible_euler_2d.jl:116-145, 3d.jl:127-150 */
typedef enum tg_source {
  TG_SOURCE_NONE = 0,
  TG_SOURCE_CONVERGENCE_TEST = 1
} tg_source;

/* TG_PRECISION_FP64: every operation in FP64 (the reference's Float64 run).
 * TG_PRECISION_MIXED: fluxes, volume/surface integrals and the 2N register
 * u_tmp in FP32; the solution u is stored as float-float pairs (hi, lo), about
 * 48 significant bits with FP32's exponent range, and its stage accumulation
 * is a float-float addition (a deviation from FP64 storage: GB300's FP64 rate
 * made even per-node FP64 conversions the bottleneck); the time, the step
 * size and all integrals stay FP64.  States cross the ABI in FP64. */
typedef enum tg_precision {
  TG_PRECISION_FP64 = 0,
  TG_PRECISION_MIXED = 1
} tg_precision;

/* Mesh of a context: TreeMesh (Cartesian elements, per-element Jacobian) or a
 * curvilinear StructuredMesh / P4estMesh brick (per-node metric terms). */
typedef enum tg_mesh_type {
  TG_MESH_TREE = 0,
  TG_MESH_CURVED = 1
} tg_mesh_type;

/* Boundary conditions of a non-periodic TreeMesh, per direction:
 * BoundaryConditionDirichlet(initial_condition) (src/equations/equations.jl:
 * 159-182) and boundary_condition_slip_wall (compressible_euler_2d.jl:322-393,
 * 3d.jl:315-416). */
typedef enum tg_boundary {
  TG_BOUNDARY_PERIODIC = 0,
  TG_BOUNDARY_DIRICHLET = 1,
  TG_BOUNDARY_SLIP_WALL = 2
} tg_boundary;

/* Initial conditions a Dirichlet boundary can take its values from, with
 * their free constants (boundary_value_params): convergence_test,
 * weak_blast_wave, constant (compressible_euler_{2,3}d.jl);
 * isentropic_vortex {p_inf, amplitude}, kelvin_helmholtz,
 * taylor_green_vortex {Ma} (the elixirs of that name); gaussian_blast
 * {p_background, energy, width}. */
typedef enum tg_initial_condition {
  TG_IC_CONSTANT = 0,
  TG_IC_CONVERGENCE_TEST = 1,
  TG_IC_ISENTROPIC_VORTEX = 2,
  TG_IC_WEAK_BLAST_WAVE = 3,
  TG_IC_KELVIN_HELMHOLTZ = 4,
  TG_IC_TAYLOR_GREEN = 5,
  TG_IC_GAUSSIAN_BLAST = 6
} tg_initial_condition;

typedef struct tg_config {
  int32_t ndims;            /* 2 or 3 */
  int32_t polydeg;          /* 1..7 (LobattoLegendreBasis) */
  int64_t nelements;        /* nelements(dg, cache) */
  int64_t ninterfaces;      /* ninterfaces(dg, cache) */
  double gamma;             /* CompressibleEulerEquations{2,3}D(gamma) */
  int32_t volume_integral;  /* tg_volume_integral */
  int32_t volume_flux;      /* tg_flux: volume_flux / volume_flux_dg */
  int32_t surface_flux;     /* tg_flux */
  int32_t volume_flux_fv;   /* tg_flux: HG low-order flux (LLF variants) */
  double alpha_max;         /* IndicatorHennemannGassner(alpha_max, alpha_min, */
  double alpha_min;         /*   alpha_smooth, variable = density_pressure)     */
  int32_t alpha_smooth;
  int32_t source_terms;     /* tg_source */
  int32_t precision;        /* tg_precision */
  int32_t device;           /* CUDA device ordinal */
  /* dg.basis (LobattoLegendreBasis): vectors of length n = polydeg + 1 and
   * n x n matrices in Julia's column-major order */
  const double* nodes;
  const double* weights;
  const double* inverse_weights;
  const double* derivative_hat;
  const double* derivative_split;
  const double* inverse_vandermonde_legendre;
  /* cache.interfaces / cache.elements (containers_{2,3}d.jl) */
  const int64_t* neighbor_ids;     /* [2, ninterfaces], 1-based element ids */
  const int64_t* orientations;     /* [ninterfaces], 1..ndims */
  const double* inverse_jacobian;  /* [nelements] */
  const double* node_coordinates;  /* [ndims, n^ndims, nelements]; may be NULL
                                      when source_terms == TG_SOURCE_NONE */
  int32_t elements_per_block;      /* 0 = library default */
  /* Non-periodic meshes (TreeMesh periodicity = false): the boundary
   * condition of each direction (-x, +x, -y, +y[, -z, +z]), applied on the
   * element faces that no interface covers; all TG_BOUNDARY_PERIODIC (0)
   * for periodic meshes.  Dirichlet faces take the values of
   * boundary_value_function (tg_initial_condition) with its free constants
   * boundary_value_params at the boundary node and the stage time; they need
   * node_coordinates. */
  int32_t boundary_conditions[6];
  int32_t boundary_value_function;
  double boundary_value_params[4];
  /* Non-conforming meshes (TreeMesh with refinement patches): the L2 mortars
   * of cache.mortars (containers_2d.jl:604-810, containers_3d.jl:591-790) and
   * the projections of dg.mortar (LobattoLegendreMortarL2,
   * basis_lobatto_legendre.jl:159-205).  nmortars = 0 (pointers may be NULL)
   * on conforming meshes.  The face of a large element towards its
   * 2^(ndims-1) small neighbours, and their faces towards it, take the
   * fluxes of prolong2mortars! / calc_mortar_flux! /
   * mortar_fluxes_to_elements! (dg_2d.jl:899-1243, dg_3d.jl:770-1335). */
  int64_t nmortars;
  const int64_t* mortar_neighbor_ids;  /* [2^(ndims-1) + 1, nmortars], 1-based:
                                          the small elements, then the large one */
  const int64_t* mortar_large_sides;   /* [nmortars]: 1 = large element on the
                                          negative side, 2 = positive side */
  const int64_t* mortar_orientations;  /* [nmortars], 1..ndims */
  const double* mortar_forward_upper;  /* n x n, column-major (as the basis) */
  const double* mortar_forward_lower;
  const double* mortar_reverse_upper;
  const double* mortar_reverse_lower;
  /* Curvilinear meshes (mesh_type = TG_MESH_CURVED): 2D StructuredMesh, and
   * P4estMesh built from a brick of trees with a uniform refinement level
   * (src/meshes/structured_mesh.jl, p4est_mesh.jl:189-244, connectivity
   * :1149-1240).  Every face is conforming and both elements of an interface
   * index its nodes in the same direction (no flipped faces); neighbor_ids /
   * orientations list each interface once as (element on the negative side,
   * element on the positive side, reference direction 1 or 2).
   * contravariant_vectors is cache.elements.contravariant_vectors
   * ([2, 2, n, n, nelements], Ja^i_x / Ja^i_y, containers_2d.jl:107-134) and
   * inverse_jacobian then points to the per-node
   * cache.elements.inverse_jacobian ([n, n, nelements], :136-152).
   * node_coordinates is [2, n, n, nelements].  Edges of the brick are periodic
 * or take TG_BOUNDARY_DIRICHLET (slip walls are not built for these meshes).
 * 3D StructuredMesh (FP64, weak form or flux differencing, polydeg 3 or 5;
 * dgsem_structured/dg_3d.jl,
 * containers_3d.jl:67-286): contravariant_vectors [3, 3, n, n, n, nelements]
 * in the curl form, inverse_jacobian [n, n, n, nelements], node_coordinates
 * [3, n, n, n, nelements], reference directions 1..3. */
  int32_t mesh_type;                   /* tg_mesh_type; 0 = TreeMesh */
  const double* contravariant_vectors;
} tg_config;

typedef struct tg_ctx tg_ctx;

int tg_api_version(void);

/* Builds a device context for one semidiscretization.  Replaces the device
 * side of create_cache (src/solvers/dgsem_tree/dg_2d.jl:14-37): copies the
 * basis and connectivity to HBM and allocates state/stage buffers. */
int tg_ctx_create(const tg_config* cfg, tg_ctx** out);
int tg_ctx_destroy(tg_ctx* ctx);

/* Message of the last failed call on ctx (ctx == NULL: last failed
 * tg_ctx_create or tg_integrals_noalloc of this thread).  Always
 * NUL-terminates when len > 0. */
int tg_last_error(const tg_ctx* ctx, char* buf, size_t len);

/* ndofs(mesh, dg, cache) (dg.jl:969-971) and ndofs * nvariables. */
int tg_ndofs(const tg_ctx* ctx, int64_t* ndofs, int64_t* nvalues);

/* Host <-> device copies of the solution (compute_coefficients! output,
 * dg.jl:1280-1325, in Trixi's layout).  Download synchronises. */
int tg_upload_state(tg_ctx* ctx, const double* u_host);
int tg_download_state(tg_ctx* ctx, double* u_host);

/* Host transfers that overlap the time stepping: the copies run on the
 * context's two copy streams (one per direction, through two FP64 device
 * staging slots each) while its own stream computes.  Host buffers are in
 * Trixi's layout, should be page-locked (pageable memory works but does not
 * overlap), and must stay valid until the transfer has completed.
 *   tg_prefetch_state  starts copying u_host into staging slot 0 or 1 and
 *                      returns at once (it waits, on the device, until the
 *                      slot's previous contents were loaded);
 *   tg_load_prefetched makes the slot's state the context's state, in the
 *                      order of the calls that enqueue work on the context
 *                      (a following tg_step uses it; the device waits for
 *                      the copy, the host does not);
 *   tg_fetch_state     enqueues the copy of the current state to u_host
 *                      through staging slot 0 or 1 and returns at once;
 *   tg_transfer_wait   blocks until the slot's prefetch copy (direction 0)
 *                      or fetch (direction 1) has completed;
 *   tg_transfer_join   makes the context stream wait for every transfer
 *                      issued so far (work enqueued after it starts when
 *                      they are done). */
int tg_prefetch_state(tg_ctx* ctx, int32_t slot, const double* u_host);
int tg_load_prefetched(tg_ctx* ctx, int32_t slot);
int tg_fetch_state(tg_ctx* ctx, int32_t slot, double* u_host);
int tg_transfer_wait(tg_ctx* ctx, int32_t slot, int32_t direction);
int tg_transfer_join(tg_ctx* ctx);

/* Device pointer of the current solution buffer.  The solution ping-pongs
 * between two buffers during tg_rk_stage/tg_step: query again after them.
 * The state may be written through it until then; the per-node indicator
 * input that mixed 2D shock-capturing stage kernels keep for the next stage
 * (rho*p of their output) is recomputed by the next tg_step or tg_rk_stage. */
int tg_state_device_ptr(tg_ctx* ctx, double** u_dev);

/* rhs_hyperbolic!(du, u, t): du and u are DEVICE pointers in Trixi's layout
 * (for instance the context state, or buffers of the caller's own).  du must
 * not alias u.  Asynchronous on the context stream. */
int tg_rhs(tg_ctx* ctx, double* du_dev, const double* u_dev, double t);

/* Same with HOST buffers: uploads u, evaluates, downloads du (synchronous). */
int tg_rhs_host(tg_ctx* ctx, double* du_host, const double* u_host, double t);

/* max_dt(u, t, mesh, constant_speed = False, equations, dg, cache) without
 * the CFL factor; u_dev == NULL uses the context state.  Synchronous. */
int tg_max_dt(tg_ctx* ctx, const double* u_dev, double* dt);

/* One fused stage of CarpenterKennedy2N54 on the context state at time t
 * with step dt (methods_2N.jl:146-158): du = rhs(u, t + c_s dt);
 * u_tmp = du - a_s u_tmp; u = u + b_s dt u_tmp.  stage = 0..4; stage 0
 * zeroes u_tmp first.  du never leaves the chip.  Asynchronous. */
int tg_rk_stage(tg_ctx* ctx, int32_t stage, double t, double dt);

/* The passes of one tg_rk_stage launched separately, so that each can be
 * timed alone: parts = 1 sets the stage clock and runs the shock indicator
 * of the current state (nothing else for contexts without HG shock
 * capturing); parts = 2 runs the element kernel of the stage (with its
 * mortar and boundary pre-passes) on the blending factors of the last
 * indicator pass and advances the state; parts = 3 is tg_rk_stage.  Part 1
 * must precede part 2 of the same stage.  No counterpart in the reference
 * (its rhs! is one call); asynchronous. */
int tg_rk_stage_part(tg_ctx* ctx, int32_t stage, double t, double dt, int32_t parts);

/* Device vectors for callers that keep the ODE state themselves: the Julia
 * shim's GB300Array, through which OrdinaryDiffEq's integrator holds u and
 * its stage registers (du, tmp) in device memory.  No counterpart in the
 * reference, whose state vectors are Julia Arrays.
 *   tg_vector_create: n FP64 values (zeroed), owned by the library until
 *     tg_vector_destroy or tg_ctx_destroy;
 *   tg_vector_copy: n values, kind 0 host -> device, 1 device -> host,
 *     2 device -> device (host transfers are synchronous);
 *   tg_lincomb: out = a x + b y elementwise (y == NULL: out = a x), out may
 *     alias x or y, asynchronous on the context stream: the broadcasts of a
 *     2N low-storage Runge-Kutta step (OrdinaryDiffEqLowStorageRK's
 *     CarpenterKennedy2N54: tmp = A tmp + dt du; u = u + B tmp). */
int tg_vector_create(tg_ctx* ctx, int64_t n, double** dev);
int tg_vector_destroy(tg_ctx* ctx, double* dev);
int tg_vector_copy(tg_ctx* ctx, void* dst, const void* src, int64_t n, int32_t kind);
int tg_lincomb(tg_ctx* ctx, int64_t n, double* out, double a, const double* x, double b,
               const double* y);

/* Time stepping with Trixi's SimpleIntegrator2N + StepsizeCallback(cfl)
 * semantics: dt = cfl * max_dt(u) after every step (and before the first
 * one), clamped to reach t_end exactly (limit_dt!).  Steps are CUDA-graph
 * launches with t, dt and the CFL reduction kept on the device; the host
 * only polls for the end.  *t_inout is the start time on entry (used on the
 * first call after an upload or tg_set_time) and the reached time on exit.
 * Stops after max_steps steps or at t_end.  Returns TG_ERR_NUMERICAL if dt
 * became NaN. */
int tg_step(tg_ctx* ctx, int64_t max_steps, double cfl, double t_end, double* t_inout,
            int64_t* steps_taken);

/* tg_step without waiting: enqueues nsteps step graphs (the same stepping,
 * stopping at t_end on the device; t_start is used as tg_step uses *t_inout)
 * and returns at once.  tg_clock_read then synchronises and reports the
 * reached time, the step count since the clock was set up and whether t_end
 * was reached (TG_ERR_NUMERICAL if dt became NaN). */
int tg_step_enqueue(tg_ctx* ctx, int64_t nsteps, double cfl, double t_end, double t_start);
int tg_clock_read(tg_ctx* ctx, double* t, int64_t* steps, int32_t* finished);

/* Resets the device clock to t (next tg_step recomputes dt). */
int tg_set_time(tg_ctx* ctx, double t);

/* FP64 domain integrals of the context state (integrate_via_indices without
 * normalisation): out[0..nvar-1] = totals of the conserved variables,
 * out[nvar] = total mathematical entropy, out[nvar+1] = kinetic energy. */
int tg_integrals(tg_ctx* ctx, double* out);

/* calc_error_norms(u, t, analyzer, semi, ...) (analysis_dg2d.jl:95-139,
 * analysis_dg3d.jl:123-...) of u_dev (an FP64 device state in Trixi's layout;
 * NULL: the context state) against the initial condition `ic`
 * (tg_initial_condition, free constants `params[4]`, may be NULL) at time t,
 * on the analyzer of Trixi's LobattoLegendreAnalyzer: its nanalyzer nodes'
 * interpolation matrix (column-major [nanalyzer, polydeg + 1], as
 * analyzer.vandermonde) and weights.  l2[nvar], linf[nvar] receive the L2
 * error (normalised by the mesh volume) and the maximum error per conserved
 * variable.  FP64 on the device, deterministic reduction; TreeMesh contexts
 * created with node coordinates.  Synchronous. */
int tg_error_norms(tg_ctx* ctx, const double* u_dev, double t, int32_t ic, const double* params,
                   int32_t nanalyzer, const double* analyzer_vandermonde,
                   const double* analyzer_weights, double* l2, double* linf);

/* analyze(entropy_timederivative, du, u, t, ...) (analysis_dg2d.jl:460-472):
 * the volume-normalised integral of cons2entropy(u) . du with du = rhs(u, t)
 * of the context state, evaluated by the context's own rhs! (FP64 or mixed)
 * and integrated in FP64.  Synchronous. */
int tg_entropy_timederivative(tg_ctx* ctx, double t, double* out);

/* Blending factors of IndicatorHennemannGassner (after smoothing) for u_dev
 * (NULL: the context state), written to alpha_host[nelements].  Synchronous.
 * Only for TG_VOLUME_SHOCK_CAPTURING_HG contexts. */
int tg_alpha(tg_ctx* ctx, const double* u_dev, double* alpha_host);

/* Refinement tree of a TreeMesh on the host (no GPU needed): Trixi's
 * TreeMesh(coordinates_min, coordinates_max; initial_refinement_level,
 * periodicity, refinement_patches) (tree_mesh.jl:128-215) with refine!
 * (2:1 rebalancing), coarsen! and the mesh containers of its leaves
 * (abstract_tree.jl:317-618, containers_{2,3}d.jl), for meshes with
 * refinement patches or AMR.  Elements are the leaves in Trixi's order.
 *   tg_tree_refine_patch: type 0 = box (a = coordinates_min, b =
 *     coordinates_max), 1 = sphere (a = center, radius).
 *   tg_tree_elements: level and cell centre ([nelements][ndims]) per element.
 *   tg_tree_interfaces / tg_tree_mortars: cache.interfaces and
 *     cache.mortars (1-based; layouts as in tg_config), sized by
 *     tg_tree_counts.
 *   tg_tree_adapt: the refine-then-coarsen pass of AMR (amr.jl:244-392) for
 *     controller values per element (+1 refine, -1 coarsen, 0 keep);
 *     changed = 0 when the mesh stayed the same.  tg_tree_transfer_map then
 *     gives the source_element / kind arrays tg_adapt_state takes.
 * Errors are read with tg_last_error(NULL, ...). */
typedef struct tg_tree tg_tree;
int tg_tree_create(int32_t ndims, int32_t initial_refinement_level, const double* coordinates_min,
                   const double* coordinates_max, const int32_t* periodicity, tg_tree** out);
int tg_tree_destroy(tg_tree* tree);
int tg_tree_refine_patch(tg_tree* tree, int32_t type, const double* a, const double* b,
                         double radius);
int tg_tree_nelements(const tg_tree* tree, int64_t* nelements);
int tg_tree_elements(const tg_tree* tree, int32_t* levels, double* centers);
int tg_tree_counts(tg_tree* tree, int64_t* ninterfaces, int64_t* nmortars);
int tg_tree_interfaces(tg_tree* tree, int64_t* neighbor_ids, int64_t* orientations);
int tg_tree_mortars(tg_tree* tree, int64_t* neighbor_ids, int64_t* large_sides,
                    int64_t* orientations);
int tg_tree_adapt(tg_tree* tree, const int8_t* controller_value, int32_t only_refine,
                  int32_t only_coarsen, int32_t* changed);
int tg_tree_transfer_map(const tg_tree* tree, int64_t* source_element, int8_t* kind);

/* AMR (AMRCallback on a TreeMesh, src/callbacks_step/amr.jl:244-392).
 *
 * tg_amr_indicator: IndicatorHennemannGassner of the context state with the
 * given parameters and indicator variable (tg_indicator_variable;
 * indicators.jl:114-148 and apply_smoothing!), always evaluated in FP64 -- the element values
 * ControllerThreeLevel compares with its thresholds (amr.jl:1116-1168).
 * Synchronous; alpha_host has nelements entries.
 *
 * tg_adapt_state: the solution transfer of refine!/coarsen!
 * (amr_dg2d.jl:85-485, amr_dg3d.jl) from the state of `src` (the mesh before
 * adaptation) into `dst` (a context built for the adapted mesh), on the
 * device.  Per new element e: kind[e] = 0 copies element source_element[e];
 * kind[e] = 1 + q makes it child q (child order of the tree, x fastest) of
 * the refined element source_element[e] by tensor-product interpolation with
 * forward_{lower,upper}; kind[e] = -1 makes it the parent of the coarsened
 * elements source_element[e] .. + 2^ndims - 1 by the sum of their
 * reverse_{lower,upper} L2 projections.  The matrices are those of the
 * LobattoLegendreAdaptorL2 (= the mortar matrices), n x n column-major.
 * Both contexts must share device, ndims, polydeg and precision.
 * Synchronous; dst then holds an uploaded state. */
typedef enum tg_indicator_variable {
  TG_INDICATOR_DENSITY_PRESSURE = 0, /* density_pressure (compressible_euler_2d.jl:2205) */
  TG_INDICATOR_DENSITY = 1           /* density */
} tg_indicator_variable;
int tg_amr_indicator(tg_ctx* ctx, double alpha_max, double alpha_min, int32_t alpha_smooth,
                     int32_t variable, double* alpha_host);
/* IndicatorMax(semi; variable) (indicators_3d.jl:239-259): the maximum of
 * the variable over the nodes of each element, FP64.  Synchronous. */
int tg_amr_indicator_max(tg_ctx* ctx, int32_t variable, double* out_host);
int tg_adapt_state(tg_ctx* dst, tg_ctx* src, const int64_t* source_element, const int8_t* kind,
                   const double* forward_upper, const double* forward_lower,
                   const double* reverse_upper, const double* reverse_lower);

/* Sticky device status word (bit 0: NaN in the state, bit 1: non-positive
 * density or pressure seen by the CFL reduction).  Reading clears it. */
int tg_status(tg_ctx* ctx, int32_t* flags);

int tg_synchronize(tg_ctx* ctx);

/* The context's CUDA stream (a cudaStream_t), for callers that order their
 * own work or timing events with the library's launches. */
int tg_stream(tg_ctx* ctx, void** stream);

/* FMA issue rate of the current device in FP32 (fp64 = 0) or FP64 (fp64 = 1),
 * in flop/s (an FMA counts two): independent FMA chains on a full-occupancy
 * grid, timed with CUDA events (a few milliseconds).  The compute-side
 * denominator for the element kernels' arithmetic rate; no counterpart in the
 * reference.  Synchronous. */
int tg_fma_peak(int32_t fp64, double* flops_per_second);

/* Allocation-free variant of tg_integrals, for callers that cannot allocate
 * device memory (a fixed-size memory pool, a runtime that owns all device
 * memory, work recorded while allocation is forbidden) and so cannot create a
 * context.  It has no counterpart in the reference.  Computes the same FP64
 * integrals (conserved totals, entropy, kinetic energy; ndims + 4 values) of
 * an FP64 state u_dev in Trixi's layout, with the element inverse Jacobians
 * inverse_jacobian_dev[nelements] and the LGL weights weights[polydeg + 1]
 * (host array), into out_dev on `stream` (a cudaStream_t; NULL = legacy
 * default stream), asynchronously.  It calls no cudaMalloc/cudaFree: its
 * scratch is a 4 MiB static device array, which limits nelements to
 * 4,194,304 (larger meshes are rejected with TG_ERR_INVALID_ARGUMENT and a
 * message for tg_last_error(NULL, ...)).  The first call on a device resolves
 * the array's device address; make that first call before any stream
 * capture.  The address is resolved again when a later call runs under a
 * different current context (after cudaDeviceReset, or with a non-primary
 * context); that call too belongs outside a capture.  All calls share the
 * array, so calls that overlap on the GPU (for example on two streams at
 * once) race. */
int tg_integrals_noalloc(int32_t ndims, int32_t polydeg, int64_t nelements, double gamma,
                         const double* weights, const double* u_dev,
                         const double* inverse_jacobian_dev, double* out_dev, void* stream);

/* ---- Learned shock indicator ----------------------------------------------
 * A small MLP (2D polydeg 3: 16 -> 64 -> 64 -> 1; 3D: 64 -> 128 -> 128 -> 1,
 * ReLU, BF16 weights, FP32 accumulation) predicting sqrt of the
 * Hennemann-Gassner smoothness indicator E of an element from its modal
 * coefficients of density*pressure normalised to unit energy
 * (indicators_2d.jl:30-101).  Deployed in place of IndicatorHennemannGassner
 * for TG_VOLUME_SHOCK_CAPTURING_HG contexts; the HG indicator stays as
 * fallback (elements whose prediction is within `band` of sqrt of the
 * switching threshold, or whose nodal density*pressure is not positive) and
 * as the judge of its error.  No counterpart in the reference, which has no
 * learned indicator. */
typedef struct tg_mlp tg_mlp;
int tg_mlp_create(int32_t ndims, int32_t polydeg, int32_t hidden, uint64_t seed, tg_mlp** out);
int tg_mlp_destroy(tg_mlp* m);
int tg_mlp_nparams(const tg_mlp* m, int64_t* n);
/* FP32 master parameters, layout W1[H][NM], b1[H], W2[H][H], b2[H], w3[H], b3. */
int tg_mlp_get_params(tg_mlp* m, float* host);
int tg_mlp_set_params(tg_mlp* m, const float* host);
/* Appends the (features, sqrt E) pairs of every stride-th element of the
 * context's current state to the network's training set. */
int tg_mlp_harvest(tg_mlp* m, tg_ctx* c, int32_t stride, int32_t phase, int64_t* total);
int tg_mlp_dataset(tg_mlp* m, float* x_host, float* y_host);
/* Adam on the mean squared error of sqrt E, minibatches drawn with
 * replacement; rows i with i % holdout == 0 are held out (holdout > 1). */
int tg_mlp_train(tg_mlp* m, int64_t steps, int32_t batch, float lr, int32_t holdout,
                 uint64_t seed, float* mean_loss);
/* Gradient of the MSE over explicit rows (for checks against a CPU oracle). */
int tg_mlp_gradient(tg_mlp* m, const float* x_host, const float* y_host, int32_t n,
                    float* grad_host, float* loss_host);
int tg_mlp_predict(tg_mlp* m, const float* x_host, int64_t n, float* pred_host);
/* Use m as the context's shock indicator (m == NULL: back to HG). */
int tg_ctx_set_learned_indicator(tg_ctx* ctx, tg_mlp* m, float band);
/* Diagnostics of the last indicator evaluation and running fallback counts
 * {elements evaluated, band fallbacks, positivity fallbacks}. */
int tg_mlp_last(tg_mlp* m, float* pred, float* hg, int32_t* flag, uint64_t* counts);

/* ---- Batched ensembles ------------------------------------------------------
 * Many independent 2D meshes of uneven sizes and polynomial degrees, advanced
 * together.  No single counterpart in the reference, where each elixir is its
 * own semidiscretize + solve (semidiscretization.jl:129-151,
 * methods_2N.jl:95-168); every instance follows exactly that.  All instances
 * are 2D, polydeg 2..4, TG_PRECISION_MIXED, with the same volume integral
 * (weak form or flux differencing), fluxes and device.  Each 2N stage of all
 * instances is one persistent kernel launch over (instance, element block)
 * work items, and each step of all instances (per-instance clocks included)
 * is one CUDA graph. */
typedef struct tg_ensemble tg_ensemble;

/* threads_per_block: 0 (default, 120), 120 or 240 (multiples of 120 fill a
 * block with whole elements for every polydeg 2..4). */
int tg_ensemble_create(const tg_config* cfgs, int32_t n, int32_t threads_per_block,
                       tg_ensemble** out);
int tg_ensemble_destroy(tg_ensemble* ens);
int tg_ensemble_size(const tg_ensemble* ens);
/* Instance i's context, owned by the ensemble: upload, download, integrals,
 * rhs and the other per-context calls work on it as usual. */
int tg_ensemble_context(tg_ensemble* ens, int32_t i, tg_ctx** ctx);
/* tg_step for every instance at once: instance i advances from t[i] (used on
 * the first step after an upload) with its own StepsizeCallback dt until
 * t_end or max_steps steps; t[i] and steps[i] (may be NULL) receive each
 * instance's reached time and step count. */
int tg_ensemble_step(tg_ensemble* ens, int64_t max_steps, double cfl, double t_end, double* t,
                     int64_t* steps);
/* Autotuner: times one stage of all instances for every block size the
 * ensemble kernel is built for (iters launches each, on the current states,
 * without changing the solution) and keeps the fastest. */
int tg_ensemble_autotune(tg_ensemble* ens, int32_t iters, int32_t* threads_per_block,
                         double* ms_per_stage);
int tg_ensemble_threads_per_block(const tg_ensemble* ens);
/* Message of the last failed call on `ens` (ens == NULL: of a failed
 * tg_ensemble_create on this thread). */
int tg_ensemble_last_error(const tg_ensemble* ens, char* buf, size_t len);

/* Elements per CUDA block in use (set by tg_config.elements_per_block or the
 * library default for the (ndims, polydeg, precision) combination). */
int tg_elements_per_block(const tg_ctx* ctx, int32_t* epb);
/* Autotuner: times one 2N stage (iters launches each) for every elements-per-
 * block value the element kernel is built with for this (ndims, polydeg) on
 * the uploaded state, without changing the solution, and keeps the fastest
 * for the following stages (best_epb, ms_per_stage may be NULL). */
int tg_ctx_autotune(tg_ctx* ctx, int32_t iters, int32_t* best_epb, double* ms_per_stage);

#ifdef __cplusplus
}
#endif

#endif /* TRIXI_GB300_H */
