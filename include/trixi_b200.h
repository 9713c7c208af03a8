/*
 * trixi_b200.h -- C ABI of libtrixi_b200.so, the GB300 (sm_103a) TreeMesh
 * DGSEM right-hand side behind TrixiCUDA.jl's public API.
 *
 * The library replaces the device side of TrixiCUDA.jl's `rhs_gpu!` path
 * (the `cuda_*` stage launchers and their CUDA.jl kernels).  Julia keeps its
 * `DGSEMGPU` / `SemidiscretizationHyperbolicGPU` / `semidiscretizeGPU` API and
 * calls these entry points with `ccall` (julia/TrixiGB300.jl holds the
 * binding).  All arrays use the reference's layouts (column-major,
 * first index fastest, integer tables 1-based Int64):
 *
 *   u, du, k             [nvars, N, (N, (N,)) nelements]           src/solvers/dg.jl:14-20
 *   interfaces u         [2, nvars, (N, (N,)) ninterfaces]         src/solvers/containers_2d.jl:58
 *   surface_flux_values  [nvars, (N, (N,)) 2*ndims, nelements]     src/solvers/containers_2d.jl:9
 *   interface neighbor_ids [2, ninterfaces], orientations [ninterfaces]
 *   mortar neighbor_ids  [2^(ndims-1)+1, nmortars]: small elements
 *                        (2D: lower, upper; 3D: lower_left, lower_right,
 *                        upper_left, upper_right) then the large element;
 *                        large_sides [nmortars] (1: large element on the
 *                        left), orientations [nmortars]
 *
 * Conventions.
 *  - Every function returns a trixi_status (0 = TRIXI_OK).  No exceptions or
 *    aborts cross the ABI.  trixi_last_error() describes the last failure.
 *  - Device pointers (u, du, k, alpha) are owned by the caller (a Julia
 *    CuArray or a torch tensor) and must live on the handle's device.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  All compute calls are asynchronous on that stream; create and
 *    destroy are synchronous.
 *  - A handle is bound to the device current at trixi_create and is not
 *    thread-safe; distinct handles may be used concurrently.
 *  - No compute call allocates device memory after the first call that
 *    needs a given buffer (the reference allocates per call,
 *    src/solvers/dg_2d.jl:349,610).
 */
#ifndef TRIXI_B200_H
#define TRIXI_B200_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TRIXI_ABI_VERSION 1

typedef struct trixi_handle trixi_handle;

typedef enum trixi_status {
  TRIXI_OK = 0,
  TRIXI_ERR_INVALID_ARGUMENT = 1, /* null/misaligned pointer, bad size, bad enum */
  TRIXI_ERR_UNSUPPORTED = 2,      /* (ndims, polydeg, equation, flux) not built */
  TRIXI_ERR_CUDA = 3,             /* a CUDA runtime call failed */
  TRIXI_ERR_DEVICE_FLAG = 4,      /* a kernel raised the device-side error word */
  TRIXI_ERR_TIMEOUT = 5,          /* a bounded device wait ran out */
  TRIXI_ERR_OUT_OF_MEMORY = 6,
  TRIXI_ERR_BAD_CONNECTIVITY = 7  /* connectivity tables inconsistent */
} trixi_status;

typedef enum trixi_equation_kind {
  TRIXI_EQ_LINEAR_ADVECTION = 0,   /* LinearScalarAdvectionEquation{1,2,3}D */
  TRIXI_EQ_COMPRESSIBLE_EULER = 1, /* CompressibleEulerEquations{1,2,3}D */
  TRIXI_EQ_IDEAL_GLM_MHD = 2       /* IdealGlmMhdEquations{1,2,3}D: 8 variables in 1D, 9 (with psi) in 2D/3D */
} trixi_equation_kind;

typedef enum trixi_volume_integral_kind {
  TRIXI_VOLUME_WEAK_FORM = 0,            /* VolumeIntegralWeakForm */
  TRIXI_VOLUME_FLUX_DIFFERENCING = 1,    /* VolumeIntegralFluxDifferencing(volume_flux) */
  TRIXI_VOLUME_SHOCK_CAPTURING_HG = 2    /* VolumeIntegralShockCapturingHG(indicator; dg, fv) */
} trixi_volume_integral_kind;

typedef enum trixi_flux_kind {
  TRIXI_FLUX_LAX_FRIEDRICHS = 0,        /* flux_lax_friedrichs, Davis wave speed max(|v|+c) */
  TRIXI_FLUX_RANOCHA = 1,               /* flux_ranocha */
  TRIXI_FLUX_CENTRAL = 2,               /* flux_central */
  TRIXI_FLUX_LAX_FRIEDRICHS_NAIVE = 3,  /* LLF with max(|v_ll|,|v_rr|) + max(c_ll,c_rr) */
  TRIXI_FLUX_HINDENLANG_GASSNER = 4,    /* flux_hindenlang_gassner (ideal GLM-MHD) */
  TRIXI_FLUX_SHIMA_ETAL = 5,            /* flux_shima_etal (Euler; a volume flux) */
  TRIXI_FLUX_HLL = 6,                   /* flux_hll: HLL with the naive min/max wave-speed estimates */
  TRIXI_FLUX_HLLE = 7                   /* flux_hlle: HLL with Einfeldt's wave speeds (Euler, ideal GLM-MHD) */
} trixi_flux_kind;

/* The nonconservative half of a (flux, nonconservative_flux) pair.  Ideal
 * GLM-MHD in 2D/3D has nonconservative terms and pairs every volume, surface
 * and FV flux with flux_nonconservative_powell (the reference's
 * noncons_volume_flux_kernel!, surface_noncons_flux_kernel!,
 * mortar_flux_kernel!: src/solvers/dg_2d_kernel.jl:228-367, 958-1035,
 * 1290-1345); every other system has none. */
typedef enum trixi_nonconservative_kind {
  TRIXI_NONCONSERVATIVE_NONE = 0,
  TRIXI_NONCONSERVATIVE_POWELL = 1  /* flux_nonconservative_powell */
} trixi_nonconservative_kind;

typedef enum trixi_precision_kind {
  TRIXI_PRECISION_FP64 = 0,  /* everything in FP64 */
  TRIXI_PRECISION_MIXED = 1  /* rhs in FP32, RK state and mortar projections in FP64 */
} trixi_precision_kind;

/* Problem description: the fields of DGSEMGPU + SemidiscretizationHyperbolicGPU
 * plus the connectivity containers built by Trixi's init_* functions
 * (src/solvers/cache.jl:60-88, src/solvers/containers_{1,2,3}d.jl).  Host
 * pointers; the library copies what it needs. */
typedef struct trixi_problem_desc {
  int32_t struct_size;          /* sizeof(trixi_problem_desc) */
  int32_t ndims;                /* 1, 2, 3 */
  int32_t polydeg;              /* 1..5 */
  int32_t nvars;                /* 1 (advection), ndims+2 (Euler), 8 / 9 (ideal GLM-MHD 1D / 2D, 3D) */
  int32_t equation;             /* trixi_equation_kind */
  int32_t volume_integral;      /* trixi_volume_integral_kind */
  int32_t volume_flux;          /* DG volume flux (flux differencing / shock capturing) */
  int32_t surface_flux;         /* surface flux (interfaces, mortars) */
  int32_t volume_flux_fv;       /* FV subcell flux (shock capturing) */
  int32_t precision;            /* trixi_precision_kind */
  double gamma;                 /* Euler ratio of specific heats */
  double advection_velocity[3]; /* advection */
  double alpha_max, alpha_min;  /* IndicatorHennemannGassner */
  int32_t alpha_smooth;
  int32_t indicator_variable;   /* 0 = density_pressure, 1 = pressure */
  int64_t nelements;
  const double *inverse_jacobian;        /* [nelements] */
  int64_t ninterfaces;
  const int64_t *interface_neighbor_ids; /* [2, ninterfaces] */
  const int64_t *interface_orientations; /* [ninterfaces] */
  int64_t nboundaries;                   /* boundary faces (0: periodic TreeMesh); tables at the end */
  int64_t nmortars;
  const int64_t *mortar_neighbor_ids;    /* [2^(ndims-1)+1, nmortars] */
  const int64_t *mortar_large_sides;     /* [nmortars] */
  const int64_t *mortar_orientations;    /* [nmortars] */
  /* Optional basis overrides (NULL = computed by the library), N x N
   * column-major as in LobattoLegendreBasisGPU / MortarL2GPU
   * (src/solvers/basis_lobatto_legendre.jl:60-100, 155-173). */
  const double *weights;
  const double *derivative_split;
  const double *derivative_dhat;
  const double *inverse_vandermonde_legendre;
  const double *forward_upper, *forward_lower, *reverse_upper, *reverse_lower;
  /* Optional node coordinates [ndims, N^ndims, nelements] (elements.node_coordinates,
   * src/solvers/containers_2d.jl:7), needed by trixi_compute_coefficients and
   * trixi_calc_error_norms with an analytic reference. */
  const double *node_coordinates;
  /* Partitioned meshes: the last nghost_elements elements are ghosts (copies
   * of another rank's elements, refreshed by a halo exchange).  Their faces
   * may be left unconnected and their rhs is not meaningful. */
  int64_t nghost_elements;
  /* Non-periodic meshes and source terms: the reference's boundaries
   * container (src/solvers/containers_2d.jl) and the boundary_conditions /
   * source_terms of SemidiscretizationHyperbolicGPU
   * (src/semidiscretization/semidiscretization_hyperbolic.jl:60-87).
   * nboundaries entries: 1-based element ids; sides 1 = the element lies on
   * the boundary's left (the boundary is its upper face), 2 = on its right;
   * orientations 1..ndims.  Every boundary face gets the Dirichlet state of
   * boundary_function -- a trixi_initial_condition_kind evaluated at the face
   * node and the time of the rhs, with the first nboundary_params of
   * boundary_params (0: the defaults of trixi_compute_coefficients) -- through
   * the surface flux, as BoundaryConditionDirichlet does (ideal GLM-MHD adds
   * 0.5 Phi(u_inner, u_boundary) of the nonconservative flux on the
   * element's side; a constant state of 9 variables does not fit
   * boundary_params and is refused with TRIXI_ERR_UNSUPPORTED).  source_terms (a
   * trixi_source_terms_kind) adds a source to du after the Jacobian; its
   * parameters (c, A, L) default to the convergence test's.  Both need
   * node_coordinates. */
  const int64_t *boundary_neighbor_ids;
  const int64_t *boundary_neighbor_sides;
  const int64_t *boundary_orientations;
  int32_t boundary_function;   /* -1: no boundaries */
  int32_t source_terms;
  int32_t nboundary_params;
  int32_t nsource_params;
  double boundary_params[8];
  double source_params[3];
  /* Ideal GLM-MHD: the nonconservative flux (trixi_nonconservative_kind) and
   * the GLM cleaning speed c_h (equations.c_h; trixi_set_glm_speed changes it
   * between steps, as a GlmSpeedCallback does). */
  int32_t nonconservative_flux;
  int32_t reserved0;            /* 0 */
  double glm_speed;
} trixi_problem_desc;

/* Library version string ("trixi_b200 <semver> sm_103a"). */
const char *trixi_version(void);
int trixi_abi_version(void);

/* Builds the device-side cache.  Replaces SemidiscretizationHyperbolicGPU's
 * create_cache_gpu (src/semidiscretization/semidiscretization_hyperbolic.jl:60-87,
 * src/solvers/cache.jl:60-88) and the GPU basis of DGSEMGPU
 * (src/solvers/dgsem_gpu.jl:43-53). */
int trixi_create(const trixi_problem_desc *desc, trixi_handle **out);
int trixi_destroy(trixi_handle *h);

/* Message of the last failure of this handle (or of the calling thread when
 * h == NULL).  Always NUL-terminates; returns the status of that failure. */
int trixi_last_error(const trixi_handle *h, char *buf, size_t len);

/* du = rhs(u, t), fully fused.  Replaces rhs_gpu!(du, u, t, mesh, ...)
 * (src/solvers/dg_1d.jl:523-548, dg_2d.jl:760-790, dg_3d.jl:895-925) and its
 * ODE-level wrapper rhs_gpu!(du_ode, u_ode, semi, t) (src/solvers/solvers.jl:18-31). */
int trixi_rhs(trixi_handle *h, double *du, const double *u, double t, void *stream);

/* One 2N low-storage RK stage, fused with the rhs:
 *   k <- a*k + dt*rhs(u_in, t);  u_out <- u_in + b*k.
 * u_out must not alias u_in (neighbour traces are read from u_in).  When
 * a == 0, k is not read.  Replaces the OrdinaryDiffEq CarpenterKennedy2N54
 * broadcast update around rhs_gpu! (examples/advection_basic_1d.jl:55). */
int trixi_rk_stage(trixi_handle *h, double *u_out, const double *u_in, double *k,
                   double a, double b, double dt, double t, void *stream);

/* nsteps CarpenterKennedy2N54 steps of size dt from time t, in place in u
 * (k is the 2N register).  The stages of a step run u -> s1 -> s2 -> s1 -> s2
 * -> u through two library-owned buffers, so no copy is needed.  With
 * precision FP32-mixed (Euler and ideal GLM-MHD), each stage after the first
 * of a call reads its flux states from an FP32 copy that the previous stage
 * wrote (two more library-owned buffers); the results are the bits of the
 * same stages run one by one through trixi_rk_stage. */
int trixi_rk_steps(trixi_handle *h, double *u, double *k, double t, double dt,
                   int64_t nsteps, void *stream);

/* trixi_rk_steps on a state in host memory, for callers whose state lives on
 * the host between steps (no counterpart in the reference, whose rhs_gpu!
 * works on device arrays): copies u_in (host, the handle's state layout) to
 * a library-owned device buffer, runs nsteps CarpenterKennedy2N54 steps
 * there (the 2N register is library-owned too: a step's first stage does not
 * read it) and copies the result to u_out (host; may be u_in).  Everything
 * is enqueued on `stream`; with page-locked host buffers the call returns
 * before the copies finish (synchronise the stream before reading u_out),
 * with pageable ones the copies block.  Optional ordering hooks for several
 * calls in flight on different streams (NULL: none): `stream` waits for
 * `wait_event` (a cudaEvent_t) after the upload and before the first stage,
 * and `done_event` is recorded after the last stage, before the download.
 * Calls on the same handle share its device buffers: calls that overlap on
 * the GPU race. */
int trixi_rk_steps_host(trixi_handle *h, const double *u_in, double *u_out, double t, double dt, int64_t nsteps,
                        void *wait_event, void *done_event, void *stream);

/* Tile tuner (no counterpart in the reference).  The fused kernel's tile --
 * warps per element group and groups per block, i.e. threads per node and
 * elements per block -- is a launch parameter.  trixi_autotune times the RK
 * stage launch for every valid tile on the state u (read only; outputs go to
 * temporary buffers) and keeps the fastest for this handle; results do not
 * depend on the tile.  Synchronous.  trixi_tile reports the elements per
 * group (compile time), the tile in use, and the tuner's candidates with
 * their ms per launch (up to `max`; *count = number measured). */
int trixi_autotune(trixi_handle *h, const double *u, void *stream);
/* Sets the tile by hand (wpg warps per group, gpb groups per block, at most 16
 * warps per block); wpg = gpb = 0 restores the compile-time default. */
int trixi_set_tile(trixi_handle *h, int wpg, int gpb);
int trixi_tile(trixi_handle *h, int *epg, int *wpg, int *gpb, int *cand_wpg, int *cand_gpb, double *cand_ms,
               int64_t max, int64_t *count);

/* Sets the GLM cleaning speed c_h of an ideal GLM-MHD handle for the
 * following calls (Trixi's GlmSpeedCallback assigns equations.c_h between
 * steps; the reference's kernels read it from `equations` at every call). */
int trixi_set_glm_speed(trixi_handle *h, double c_h);

/* Stage entry points with the reference's stage split (the de-facto API used
 * by the reference tests, src/solvers/dg.jl:181-301, docs/src/reference.md:14-30).
 * They compute in FP64 and fill the library-owned containers below. */
int trixi_volume_integral(trixi_handle *h, double *du, const double *u, void *stream);  /* cuda_volume_integral! */
int trixi_prolong2interfaces(trixi_handle *h, const double *u, void *stream);          /* cuda_prolong2interfaces! */
int trixi_interface_flux(trixi_handle *h, void *stream);                               /* cuda_interface_flux! */
int trixi_prolong2boundaries(trixi_handle *h, const double *u, void *stream);          /* cuda_prolong2boundaries! (periodic: no-op) */
int trixi_boundary_flux(trixi_handle *h, double t, void *stream);                      /* cuda_boundary_flux! (periodic: no-op) */
int trixi_prolong2mortars(trixi_handle *h, const double *u, void *stream);             /* cuda_prolong2mortars! */
int trixi_mortar_flux(trixi_handle *h, void *stream);                                  /* cuda_mortar_flux! */
int trixi_surface_integral(trixi_handle *h, double *du, void *stream);                 /* cuda_surface_integral! */
int trixi_jacobian(trixi_handle *h, double *du, void *stream);                         /* cuda_jacobian! */
int trixi_sources(trixi_handle *h, double *du, const double *u, double t, void *stream); /* cuda_sources! (none: no-op) */

/* Library-owned containers (device pointers), mirroring cache_gpu fields. */
typedef enum trixi_container_id {
  TRIXI_CONTAINER_INTERFACES_U = 0,        /* cache.interfaces.u */
  TRIXI_CONTAINER_SURFACE_FLUX_VALUES = 1, /* cache.elements.surface_flux_values */
  TRIXI_CONTAINER_MORTARS_U = 2,           /* 2D: +0 u_upper, +1 u_lower; 3D: +0 u_upper_left,
                                              +1 u_upper_right, +2 u_lower_left, +3 u_lower_right */
  TRIXI_CONTAINER_ALPHA = 8,               /* shock-capturing blending factor [nelements] */
  TRIXI_CONTAINER_INVERSE_JACOBIAN = 9,
  TRIXI_CONTAINER_BOUNDARIES_U = 10        /* cache.boundaries.u [2, nvars, N^(ndims-1), nboundaries] */
} trixi_container_id;
int trixi_container(trixi_handle *h, int which, void **dev_ptr, int64_t *count);

/* Hennemann-Gassner indicator on the GPU: alpha[nelements] (device) from u,
 * smoothed as configured.  Replaces the host round trip
 * `indicator(Array(u), ...)` of src/solvers/dg_3d.jl:187 (indicators.jl:7-42). */
int trixi_indicator(trixi_handle *h, const double *u, double *alpha, void *stream);

/* Initial conditions evaluated on the GPU (params may be NULL for defaults):
 *   TRIXI_IC_CONSTANT          params = the nvars conservative values (up to 9)
 *   TRIXI_IC_CONVERGENCE_TEST  params = (c, A, L); advection default (1, 0.5, 2),
 *                              Euler default (2, 0.1, 2); ideal GLM-MHD: the
 *                              smooth Alfven waves, no params
 *   TRIXI_IC_WEAK_BLAST_WAVE   Euler, ideal GLM-MHD (in B = (1, 1, 1)); no params
 *   TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY
 *                              Euler: the manufactured solution of the
 *                              Euler-gravity convergence test,
 *                              rho = 2 + 0.1 sin(pi (sum_d x_d - t)), v_d = 1,
 *                              p = 2 G rho^2 / (ndims pi) with G = 1 (the
 *                              pressure of hydrostatic balance with the
 *                              gravitational potential of rho); no params
 *                              (test/tree_dgsem_3d/euler_convergence.jl:11) */
typedef enum trixi_initial_condition_kind {
  TRIXI_IC_CONSTANT = 0,
  TRIXI_IC_CONVERGENCE_TEST = 1,
  TRIXI_IC_WEAK_BLAST_WAVE = 2,
  TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY = 3
} trixi_initial_condition_kind;

/* Source terms (desc.source_terms), Euler only:
 *   TRIXI_SOURCE_CONVERGENCE_TEST  source_terms_convergence_test, the source of
 *       the manufactured solution rho = rho v_d = c + A sin(2 pi/L (sum_d x_d - t)),
 *       E = rho^2;
 *   TRIXI_SOURCE_EOC_TEST_EULER    source_terms_eoc_test_euler, the source that
 *       makes TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY an exact solution of the
 *       Euler equations without gravity (test/tree_dgsem_3d/euler_convergence.jl:24). */
typedef enum trixi_source_terms_kind {
  TRIXI_SOURCE_NONE = 0,
  TRIXI_SOURCE_CONVERGENCE_TEST = 1,
  TRIXI_SOURCE_EOC_TEST_EULER = 2
} trixi_source_terms_kind;

/* u = initial condition at the nodes (needs desc.node_coordinates); 1D
 * moves element end points one ulp inwards like the reference.  Replaces
 * compute_coefficients_gpu / compute_coefficients_kernel! (src/solvers/dg.jl:46-160,
 * src/semidiscretization/semidiscretization.jl:4-20). */
int trixi_compute_coefficients(trixi_handle *h, int ic_kind, const double *params, int64_t nparams, double t,
                               double *u, void *stream);

/* dt_dev[0] = 2 / (N * max_e J^{-1}_e sum_d max_nodes lambda_d(u)) on the GPU
 * (device scalar; multiply by the CFL number).  Replaces max_dt of the
 * StepsizeCallback (src/callbacks_step/stepsize_dg_{1,2,3}d.jl), which copies
 * u to the host every step. */
int trixi_max_dt(trixi_handle *h, const double *u, double *dt_dev, void *stream);

/* Quadrature integrals sum_e J_e sum_nodes w q (not normalised by the volume):
 *   TRIXI_INTEGRAL_STATE               q = u (nvars results)
 *   TRIXI_INTEGRAL_ENTROPY             q = -rho s/(gamma-1) (Euler), u^2/2 (advection)
 *   TRIXI_INTEGRAL_ENTROPY_PRODUCTION  q = w(u) . du with the entropy variables w
 *   TRIXI_INTEGRAL_DU                  q = du (nvars results)
 * Synchronous: results are written to host memory.  Replaces
 * integrate_via_indices (src/callbacks_step/analysis_dg_2d.jl:1-40). */
typedef enum trixi_integral_kind {
  TRIXI_INTEGRAL_STATE = 0,
  TRIXI_INTEGRAL_ENTROPY = 1,
  TRIXI_INTEGRAL_ENTROPY_PRODUCTION = 2,
  TRIXI_INTEGRAL_DU = 3
} trixi_integral_kind;
int trixi_integrate(trixi_handle *h, const double *u, const double *du, int which, double *out_host, int64_t count,
                    void *stream);

/* The integrals of trixi_integrate, for linear advection and compressible
 * Euler (equation TRIXI_EQ_LINEAR_ADVECTION or TRIXI_EQ_COMPRESSIBLE_EULER;
 * ideal GLM-MHD is refused with TRIXI_ERR_INVALID_ARGUMENT -- use
 * trixi_integrate), for callers that cannot allocate device memory.  No counterpart in the reference: it exists for callers whose GPU
 * memory belongs to another allocator (a CUDA.jl or PyTorch caching pool that
 * has reserved the device) and for loops that must not pay the device-wide
 * synchronisation of cudaMalloc / cudaFree.  It needs no handle and calls no
 * allocating routine: u, du (node layout [nelements][N^ndims][nvars]),
 * inverse_jacobian[nelements] and out_dev (nvars values for STATE and DU, one
 * otherwise) are device pointers owned by the caller; the per-element partial
 * sums go to a static device array of 2^20 doubles (8 MiB) that every GPU
 * loading the library reserves until the process exits.  Calls with
 * nelements * (number of results) > 2^20 return TRIXI_ERR_INVALID_ARGUMENT.
 * The first call on a device looks up that array's address with the device
 * current, so make it before any stream capture.  All calls share the array
 * and it keeps the last call's contents (each call writes every slot it
 * reads); calls whose kernels overlap on the GPU race on it.  Asynchronous on
 * `stream`; errors are read with trixi_last_error(NULL, ...). */
int trixi_integrate_noalloc(int ndims, int polydeg, int equation, double gamma, const double *u, const double *du,
                            const double *inverse_jacobian, int64_t nelements, int which, double *out_dev,
                            void *stream);

/* L2 and Linf errors per variable after interpolation to 2*polydeg+1 LGL
 * analysis nodes, against an analytic initial condition at time t (u_ref
 * NULL) or against a second state u_ref on the same mesh.  L2 is normalised
 * by the total volume.  Synchronous.  Replaces calc_error_norms
 * (src/callbacks_step/analysis_dg_2d.jl:44-89). */
int trixi_calc_error_norms(trixi_handle *h, const double *u, const double *u_ref, int ic_kind, const double *params,
                           int64_t nparams, double t, double *l2_host, double *linf_host, void *stream);

/* Copies a basis operator to host memory: 0 nodes, 1 weights, 2 derivative_split,
 * 3 derivative_dhat, 4 inverse_vandermonde_legendre, 5 forward_upper,
 * 6 forward_lower, 7 reverse_upper, 8 reverse_lower, 9 derivative_matrix. */
int trixi_basis(const trixi_handle *h, int which, double *host_out, int64_t count);

/* Same operators without a handle (pure host code, no GPU needed). */
int trixi_lgl_basis(int polydeg, int which, double *host_out, int64_t count);

/* ---- Batched ensembles (no counterpart in the reference, which solves one
 * problem at a time) --------------------------------------------------------
 * Hundreds of independent instances (mixed ndims, polydeg, equations, meshes,
 * mortars) advanced together.  Instances with the same kernel kind are merged
 * into one group whose elements are concatenated (connectivity offset), so a
 * group is served by one fused launch per RK stage; a full RK step of all
 * groups is captured as a CUDA graph.  All instances share one precision.
 * The batch state is one device buffer: instance i occupies
 * [value_offsets[i], value_offsets[i] + nvalues[i]) in its own reference
 * layout [nvars, N, .., nelements_i]; instances are ordered by group. */
typedef struct trixi_batch trixi_batch;
int trixi_batch_create(const trixi_problem_desc *const *descs, int64_t n, trixi_batch **out);
int trixi_batch_destroy(trixi_batch *b);
int trixi_batch_layout(const trixi_batch *b, int64_t *value_offsets, int64_t *nvalues, int64_t *total_values,
                       int64_t *ngroups);
int trixi_batch_rhs(trixi_batch *b, double *du, const double *u, void *stream);
/* nsteps CarpenterKennedy2N54 steps; instance i uses dt_per_instance[i] (host
 * array).  use_graph != 0 replays a captured CUDA graph of the whole step, in
 * which the groups run as parallel branches; the first graph build tunes, on
 * copies of u and k, the tile of every group's kernel (as trixi_autotune) and
 * then the branch count. */
int trixi_batch_rk_steps(trixi_batch *b, double *u, double *k, const double *dt_per_instance, int64_t nsteps,
                         int use_graph, void *stream);
/* The tuner's choice and its timings: *branches (0 before the first graph
 * build), up to `max` candidate branch counts with their ms per step, and the
 * number of candidates in *count. */
int trixi_batch_tuning(const trixi_batch *b, int *branches, int *candidates, double *ms_per_step, int64_t max,
                       int64_t *count);
/* The merged handle of one group (for the stage API and analysis calls). */
int trixi_batch_handle(trixi_batch *b, int64_t group, trixi_handle **h);
int trixi_batch_last_error(const trixi_batch *b, char *buf, size_t len);

/* ---- Discrete adjoint (no counterpart in the reference) --------------------
 * FP64; Euler flux differencing with flux_ranocha / flux_central and linear
 * advection, on conforming periodic meshes. */

/* ubar = J_rhs(u)^T lambda (device arrays in the state layout). */
int trixi_rhs_vjp(trixi_handle *h, double *ubar, const double *u, const double *lambda, void *stream);

/* J = 1/2 * sum_e J_e sum_nodes w (rho - rho_target)^2 (host scalar) and, if
 * ubar != NULL, its gradient with respect to the state (device).  rho_target
 * holds one value per node [N^ndims, nelements]. */
int trixi_objective_density_l2(trixi_handle *h, const double *u, const double *rho_target, double *J_host,
                               double *ubar, void *stream);

/* Forward sweep of nsteps CarpenterKennedy2N54 steps of size dt from u0,
 * storing up to nsnapshots checkpoints (binomial schedule); writes u(T).
 * nsnapshots >= nsteps - 1 stores every step (no recomputation). */
int trixi_adjoint_forward(trixi_handle *h, const double *u0, double dt, int64_t nsteps, int64_t nsnapshots,
                          double *uT, void *stream);

/* Backward sweep: given dJ/du(T) returns dJ/du0, recomputing states from the
 * checkpoints.  *forward_steps = RK steps recomputed (0 when all were stored). */
int trixi_adjoint_backward(trixi_handle *h, const double *uT_bar, double *u0_bar, int64_t *forward_steps,
                           void *stream);

/* Waits for the handle's stream work, then checks the device error word. */
int trixi_synchronize(trixi_handle *h, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TRIXI_B200_H */
