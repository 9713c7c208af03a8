/*
 * trixi_oracle.h -- CPU restatement of the TreeMesh DGSEM right-hand side.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the GPU library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product never links, loads or falls back to it.
 *
 * Parity status: UNPINNED at the Trixi.jl boundary.  The reference
 * (TrixiCUDA.jl) is pure Julia and takes its arithmetic from Trixi.jl, which
 * is not vendored, and neither Julia nor Trixi.jl can run here; the
 * reference ships no golden vectors.  The oracle is pinned instead by
 * analytic known answers (LGL nodes/weights, exact polynomial derivatives,
 * SBP property, exact L2 mortar projections) and by discrete invariants
 * (free-stream preservation, conservation, entropy conservation of
 * flux_ranocha, convergence order, 2N-RK order) -- see tests/.
 *
 * Array layouts follow the reference containers exactly (Julia column-major,
 * first index fastest, all integer tables 1-based Int64):
 *   u, du                [nvars, N, (N, (N,)) nelements]        src/solvers/dg.jl:14-20
 *   interfaces_u         [2, nvars, (N, (N,)) ninterfaces]      src/solvers/containers_2d.jl:58
 *   surface_flux_values  [nvars, (N, (N,)) 2*ndims, nelements]  src/solvers/containers_2d.jl:9
 *   mortar u arrays      2D: u_upper/u_lower [2, nvars, N, nmortars];
 *                        3D: u_upper_left/right, u_lower_left/right [2, nvars, N, N, nmortars]
 *                        (src/solvers/containers_2d.jl, containers_3d.jl)
 *   interface neighbor_ids [2, ninterfaces], orientations [ninterfaces]
 *   mortar neighbor_ids  [2^(ndims-1)+1, nmortars] (small..., large), large_sides, orientations
 */
#ifndef TRIXI_ORACLE_H
#define TRIXI_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_EQ_ADVECTION = 0, ORC_EQ_EULER = 1, ORC_EQ_MHD = 2 };
enum { ORC_NONCONS_NONE = 0, ORC_NONCONS_POWELL = 1 };
enum { ORC_VOL_WEAK = 0, ORC_VOL_FLUXDIFF = 1, ORC_VOL_SHOCK_HG = 2 };
enum { ORC_FLUX_LLF = 0, ORC_FLUX_RANOCHA = 1, ORC_FLUX_CENTRAL = 2, ORC_FLUX_LLF_NAIVE = 3,
       ORC_FLUX_HINDENLANG_GASSNER = 4, ORC_FLUX_SHIMA_ETAL = 5, ORC_FLUX_HLL = 6,
       ORC_FLUX_HLLE = 7 };
enum { ORC_IC_CONSTANT = 0, ORC_IC_CONVERGENCE_TEST = 1, ORC_IC_WEAK_BLAST_WAVE = 2, ORC_IC_EOC_EULER_GRAVITY = 3 };
enum { ORC_SRC_NONE = 0, ORC_SRC_CONVERGENCE_TEST = 1, ORC_SRC_EOC_EULER = 2 };

typedef struct {
  int32_t ndims, polydeg, nvars, equation;
  double gamma;
  double advection_velocity[3];
  int32_t volume_integral, volume_flux, surface_flux, volume_flux_fv;
  double alpha_max, alpha_min;
  int32_t alpha_smooth;
  int64_t nelements, ninterfaces, nmortars;
  const double *inverse_jacobian;           /* [nelements] */
  const int64_t *interface_neighbor_ids;    /* [2, ninterfaces], 1-based */
  const int64_t *interface_orientations;    /* [ninterfaces], 1..ndims */
  const int64_t *mortar_neighbor_ids;       /* [2^(ndims-1)+1, nmortars], 1-based */
  const int64_t *mortar_large_sides;        /* [nmortars], 1 or 2 */
  const int64_t *mortar_orientations;       /* [nmortars], 1..ndims */
  /* non-periodic meshes: the boundaries container (containers_2d.jl) and the
   * Dirichlet boundary function, an ORC_IC_* kind evaluated at (x, t) */
  int64_t nboundaries;
  const int64_t *boundary_neighbor_ids;     /* [nboundaries], 1-based */
  const int64_t *boundary_neighbor_sides;   /* [nboundaries], 1: element left of it, 2: right */
  const int64_t *boundary_orientations;     /* [nboundaries], 1..ndims */
  int32_t boundary_function;                /* ORC_IC_* */
  int32_t source_terms;                     /* ORC_SRC_* */
  double boundary_params[8];                /* constant state, or (c, A, L) of the convergence test */
  double source_params[3];                  /* (c, A, L) of the manufactured solution */
  const double *node_coordinates;           /* [ndims, N^ndims, nelements] (needed with boundaries / sources) */
  /* ideal GLM-MHD: the nonconservative flux paired with the volume and surface
   * fluxes (flux_nonconservative_powell) and the GLM cleaning speed c_h */
  int32_t nonconservative_flux;             /* ORC_NONCONS_* */
  double glm_speed;
  int32_t indicator_variable;               /* 0: density_pressure (rho p), 1: pressure */
} oracle_desc;

typedef struct oracle_handle oracle_handle;

/* Basis of N = polydeg+1 Lobatto-Legendre nodes.  Matrices are N x N,
 * column-major (M[i,j] at i + N*j), as Julia stores them. */
int oracle_basis(int polydeg, double *nodes, double *weights, double *dmat,
                 double *dsplit, double *dhat, double *inv_vandermonde,
                 double *forward_upper, double *forward_lower,
                 double *reverse_upper, double *reverse_lower);

oracle_handle *oracle_create(const oracle_desc *desc);
void oracle_destroy(oracle_handle *h);
int oracle_set_threads(int nthreads);

/* Stage functions: same stage split as the reference's cuda_* launchers. */
void oracle_volume_integral(oracle_handle *h, double *du, const double *u, const double *alpha);
void oracle_prolong2interfaces(oracle_handle *h, const double *u, double *interfaces_u);
void oracle_interface_flux(oracle_handle *h, const double *interfaces_u, double *surface_flux_values);
void oracle_prolong2mortars(oracle_handle *h, const double *u, double *const *mortar_u);
void oracle_mortar_flux(oracle_handle *h, double *const *mortar_u, double *surface_flux_values);
void oracle_surface_integral(oracle_handle *h, double *du, const double *surface_flux_values);
void oracle_jacobian(oracle_handle *h, double *du);
void oracle_indicator_hg(oracle_handle *h, const double *u, double *alpha);
void oracle_prolong2boundaries(oracle_handle *h, const double *u, double *boundaries_u);
void oracle_boundary_flux(oracle_handle *h, const double *boundaries_u, double t, double *surface_flux_values);
void oracle_sources(oracle_handle *h, double *du, double t);
/* the boundary function / initial conditions at one point */
void oracle_eval_ic(oracle_handle *h, int kind, const double *params, const double *x, double t, double *u);

/* Whole right-hand side and the CarpenterKennedy2N54 time stepper. */
void oracle_rhs(oracle_handle *h, double *du, const double *u, double t);
void oracle_rk_ck2n54(oracle_handle *h, double *u, double *k, double t, double dt, int nsteps);

/* Pointwise fluxes of the problem's equations along orientation o (0-based):
 * the physical flux, a two-point flux of kind ORC_FLUX_*, and the
 * nonconservative term Phi(u_l, u_r) (zero without one). */
void oracle_physical_flux(oracle_handle *h, const double *u, int o, double *f);
void oracle_two_point_flux(oracle_handle *h, int kind, const double *ul, const double *ur, int o, double *f);
void oracle_noncons_flux(oracle_handle *h, const double *ul, const double *ur, int o, double *f);

/* Sizes of the internal containers (for callers that want the stage arrays). */
int64_t oracle_size(oracle_handle *h, int which);

#ifdef __cplusplus
}
#endif
#endif
