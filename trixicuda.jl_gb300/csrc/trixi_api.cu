// trixi_api.cu -- the C ABI of libtrixi_b200.so (declared in include/trixi_b200.h).
//
// Host runtime: validates the problem description and connectivity, builds
// the per-element face table (one int32 per element face: the neighbour
// element, or a mortar-flux slot), uploads tables and basis operators, owns
// scratch buffers, and sequences the kernels of one rhs / RK stage on the
// caller's stream.  Every entry point returns a trixi_status; nothing throws
// across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <map>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/trixi_b200.h"
#include "basis.h"
#include "dg_adjoint.h"
#include "dg_analysis.h"
#include "dg_host.h"

using namespace trixi;

namespace {

thread_local std::string g_last_error;
thread_local int g_last_status = TRIXI_OK;

}  // namespace

void trixi::set_last_error(int status, const char *msg) {
  g_last_error = msg ? msg : "";
  g_last_status = status;
}

namespace {

// CarpenterKennedy2N54 coefficients (Carpenter & Kennedy 1994, NASA TM-109112).  The
// stage times t + c_s dt are not needed: the semidiscretization is autonomous
// (periodic boundaries, no source terms).
const double kCK_A[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                         -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
const double kCK_B[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                         2277821191437.0 / 14882151754819.0};
// stage times t + c_s dt of CarpenterKennedy2N54
const double kCK_C[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                         2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

}  // namespace

struct AdjointState {
  int64_t n = 0, snapshots = 0;
  double dt = 0.0;
  bool forward_done = false;
  int64_t fwd_steps = 0;
  double *u0 = nullptr, *ktmp = nullptr, *tmp = nullptr;
  double *stage[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double *lu[2] = {nullptr, nullptr}, *lk[2] = {nullptr, nullptr};
  std::vector<double *> pool;           // free snapshot buffers
  std::map<int64_t, double *> ckpt;     // step -> stored state
  double *stages_all = nullptr;         // store-all mode: the 5 stage inputs of every step
  std::vector<double *> all;            // every allocation, for cleanup
};

struct trixi_handle {
  int device = 0;
  int dim = 0, N = 0, nv = 0, NN = 0, NF = 0, nchild = 1;
  int eq = 0, vol = 0, vflux = 0, sflux = 0, fvflux = 0;
  bool mixed = false;
  double gamma = 1.4, adv[3] = {0, 0, 0};
  double c_h = 0.0;  // GLM cleaning speed (ideal GLM-MHD)
  double alpha_max = 0.5, alpha_min = 0.001;
  int alpha_smooth = 1;
  int ind_var = 0;  // indicator variable: 0 density_pressure, 1 pressure
  int64_t E = 0, I = 0, M = 0, B = 0;
  Basis basis;
  // non-periodic meshes and source terms
  int bc_kind = -1, src_kind = 0;
  IcParams bc{};
  double src[3] = {2.0, 0.1, 2.0};
  int64_t *d_bnd_nid = nullptr, *d_bnd_side = nullptr, *d_bnd_ori = nullptr;
  double *d_boundaries_u = nullptr;
  // device tables
  int32_t *d_face_table = nullptr;
  int32_t *d_slot_nbrs = nullptr;
  double *d_inv_jac = nullptr;
  int64_t *d_if_nid = nullptr, *d_if_ori = nullptr;
  int64_t *d_mo_nid = nullptr, *d_mo_ls = nullptr, *d_mo_ori = nullptr;
  double *d_mortar_flux = nullptr;
  double *d_alpha_raw = nullptr, *d_alpha = nullptr;
  int *d_err = nullptr;
  double *d_scratch_u = nullptr, *d_scratch_u2 = nullptr;  // RK stage buffers of trixi_rk_steps
  // FP32 copies of the stage states inside trixi_rk_steps (FP32-mixed Euler
  // and MHD): stage g reads copy g % 2 and writes copy (g + 1) % 2
  float *d_u32[2] = {nullptr, nullptr};
  double *d_host_u = nullptr, *d_host_k = nullptr;  // device state and 2N register of trixi_rk_steps_host
  // stage containers (allocated on first use)
  double *d_interfaces_u = nullptr, *d_sfv = nullptr, *d_mortar_u[4] = {nullptr, nullptr, nullptr, nullptr};
  // analysis / initial conditions (allocated on first use)
  double *d_coords = nullptr;
  unsigned long long *d_acc = nullptr;
  double *d_partial = nullptr, *d_partial2 = nullptr, *d_red_out = nullptr;
  double *d_vdm = nullptr, *d_wa = nullptr, *d_w = nullptr;
  std::vector<double> xa;
  double total_volume = 0.0;
  struct AdjointState *adj = nullptr;
  FusedHost fused;
  // tile tuner record: candidate (wpg, gpb) and ms per RK-stage launch
  std::vector<int> tune_wpg, tune_gpb;
  std::vector<double> tune_ms;
  std::string last_error;
  int last_status = TRIXI_OK;
};

namespace {

int fail(trixi_handle *h, int status, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  g_last_status = status;
  if (h) {
    h->last_error = buf;
    h->last_status = status;
  }
  return status;
}

int cuda_fail(trixi_handle *h, cudaError_t e, const char *what) {
  if (e == cudaErrorNotSupported) return fail(h, TRIXI_ERR_UNSUPPORTED, "%s: combination not compiled", what);
  if (e == cudaErrorMemoryAllocation) return fail(h, TRIXI_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  return fail(h, TRIXI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define TRIXI_CUDA(h, expr, what)                     \
  do {                                                \
    cudaError_t e_ = (expr);                          \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

bool aligned8(const void *p) { return p && ((uintptr_t)p % 8 == 0); }

template <typename T>
cudaError_t upload(T **dst, const T *src, size_t n) {
  if (n == 0) {
    *dst = nullptr;
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc((void **)dst, n * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

void free_adjoint(trixi_handle *h) {
  if (!h->adj) return;
  for (double *p : h->adj->all) cudaFree(p);
  delete h->adj;
  h->adj = nullptr;
}

void free_all(trixi_handle *h) {
  free_adjoint(h);
  void *ptrs[] = {h->d_face_table, h->d_slot_nbrs, h->d_inv_jac, h->d_if_nid, h->d_if_ori, h->d_mo_nid,
                  h->d_mo_ls, h->d_mo_ori, h->d_mortar_flux, h->d_alpha_raw, h->d_alpha, h->d_err,
                  h->d_scratch_u, h->d_scratch_u2, h->d_interfaces_u, h->d_sfv, h->d_mortar_u[0], h->d_mortar_u[1],
                  h->d_mortar_u[2], h->d_mortar_u[3], h->d_coords, h->d_acc, h->d_partial, h->d_partial2,
                  h->d_red_out, h->d_vdm, h->d_wa, h->d_w, h->d_bnd_nid, h->d_bnd_side, h->d_bnd_ori,
                  h->d_boundaries_u, h->d_u32[0], h->d_u32[1], h->d_host_u, h->d_host_k};
  for (void *p : ptrs)
    if (p) cudaFree(p);
}

// row-major copies of the column-major basis for the kernels
void to_row_major(const std::vector<double> &cm, int n, double *rm) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) rm[i * n + j] = cm[i + (size_t)n * j];
}

int64_t ipow64(int64_t b, int e) {
  int64_t r = 1;
  while (e-- > 0) r *= b;
  return r;
}

IcParams ic_params(const trixi_handle *h, int kind, const double *params, int64_t nparams);

int check_u_args(trixi_handle *h, const void *a, const char *name) {
  if (!aligned8(a)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "%s is null or not 8-byte aligned", name);
  return TRIXI_OK;
}

}  // namespace

extern "C" {

const char *trixi_version(void) { return "trixi_b200 0.1.0 sm_103a"; }
int trixi_abi_version(void) { return TRIXI_ABI_VERSION; }

int trixi_last_error(const trixi_handle *h, char *buf, size_t len) {
  const std::string &msg = h ? h->last_error : g_last_error;
  if (buf && len > 0) {
    size_t n = std::min(len - 1, msg.size());
    std::memcpy(buf, msg.data(), n);
    buf[n] = '\0';
  }
  return h ? h->last_status : g_last_status;
}

int trixi_create(const trixi_problem_desc *d, trixi_handle **out) {
  if (!out) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (!d) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "desc is null");
  if (d->struct_size != (int32_t)sizeof(trixi_problem_desc))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "desc.struct_size %d != %d", d->struct_size,
                (int)sizeof(trixi_problem_desc));
  if (d->ndims < 1 || d->ndims > 3) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "ndims %d", d->ndims);
  if (d->polydeg < 1 || d->polydeg + 1 > HOST_NMAX)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "polydeg %d (supported 1..%d)", d->polydeg, HOST_NMAX - 1);
  if (d->equation != TRIXI_EQ_LINEAR_ADVECTION && d->equation != TRIXI_EQ_COMPRESSIBLE_EULER &&
      d->equation != TRIXI_EQ_IDEAL_GLM_MHD)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "equation %d", d->equation);
  const bool mhd = d->equation == TRIXI_EQ_IDEAL_GLM_MHD;
  const int nv_expect = d->equation == TRIXI_EQ_LINEAR_ADVECTION ? 1 : mhd ? (d->ndims == 1 ? 8 : 9) : d->ndims + 2;
  if (d->nvars != nv_expect)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "nvars %d, equation needs %d", d->nvars, nv_expect);
  if (d->volume_integral < 0 || d->volume_integral > 2)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "volume_integral %d", d->volume_integral);
  for (int f : {d->volume_flux, d->surface_flux, d->volume_flux_fv})
    if (f < 0 || f > 7) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "flux enum %d", f);
  // flux_shima_etal is a volume flux (flux differencing / the DG part of shock
  // capturing); surface and FV fluxes are the runtime-selected kinds
  if (d->surface_flux == TRIXI_FLUX_SHIMA_ETAL || d->volume_flux_fv == TRIXI_FLUX_SHIMA_ETAL)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "flux_shima_etal as a surface or FV flux");
  if (d->volume_flux == TRIXI_FLUX_SHIMA_ETAL && d->equation != TRIXI_EQ_COMPRESSIBLE_EULER)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "flux_shima_etal needs the Euler equations");
  if (d->volume_flux == TRIXI_FLUX_SHIMA_ETAL && (d->nboundaries > 0 || d->source_terms != TRIXI_SOURCE_NONE))
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "flux_shima_etal: periodic meshes without source terms");
  if ((d->volume_flux == TRIXI_FLUX_HLL || d->volume_flux == TRIXI_FLUX_HLLE) &&
      d->volume_integral != TRIXI_VOLUME_WEAK_FORM)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "flux_hll / flux_hlle as a volume flux");
  if ((d->surface_flux == TRIXI_FLUX_HLLE || d->volume_flux_fv == TRIXI_FLUX_HLLE) &&
      d->equation == TRIXI_EQ_LINEAR_ADVECTION)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "flux_hlle needs the Euler or MHD equations");
  for (int f : {d->volume_flux, d->surface_flux, d->volume_flux_fv}) {
    // flux_hindenlang_gassner is the MHD flux, flux_ranocha the Euler one
    if (f == TRIXI_FLUX_HINDENLANG_GASSNER && !mhd)
      return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "flux_hindenlang_gassner needs ideal GLM-MHD");
    if (f == TRIXI_FLUX_RANOCHA && mhd)
      return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "flux_ranocha is not defined for ideal GLM-MHD");
  }
  {
    // ideal GLM-MHD in 2D/3D pairs every flux with flux_nonconservative_powell
    // (have_nonconservative_terms); every other system takes plain fluxes
    const int need = (mhd && d->ndims > 1) ? TRIXI_NONCONSERVATIVE_POWELL : TRIXI_NONCONSERVATIVE_NONE;
    if (d->nonconservative_flux != need)
      return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "nonconservative_flux %d, the equations need %d",
                  d->nonconservative_flux, need);
  }
  if (mhd && d->source_terms != TRIXI_SOURCE_NONE)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "ideal GLM-MHD: no source terms");
  if (mhd && d->nboundaries > 0 && d->boundary_function == TRIXI_IC_CONSTANT && d->nvars > 8)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "ideal GLM-MHD: a constant Dirichlet state needs 9 > 8 parameters");
  if (mhd && d->volume_integral == TRIXI_VOLUME_WEAK_FORM)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "ideal GLM-MHD: flux differencing or shock capturing");
  if (d->volume_integral == TRIXI_VOLUME_SHOCK_CAPTURING_HG && d->indicator_variable != 0 && d->indicator_variable != 1)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "indicator_variable %d", d->indicator_variable);
  if (d->precision != TRIXI_PRECISION_FP64 && d->precision != TRIXI_PRECISION_MIXED)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "precision %d", d->precision);
  if (d->nelements <= 0 || d->nelements > INT32_MAX)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "nelements %lld", (long long)d->nelements);
  if (!d->inverse_jacobian) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "inverse_jacobian is null");
  if (d->ninterfaces < 0 || (d->ninterfaces > 0 && (!d->interface_neighbor_ids || !d->interface_orientations)))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "interface tables");
  if (d->nboundaries < 0 || (d->nboundaries > 0 && (!d->boundary_neighbor_ids || !d->boundary_neighbor_sides ||
                                                    !d->boundary_orientations)))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "boundary tables");
  if (d->nboundaries > 0 && (d->boundary_function < TRIXI_IC_CONSTANT ||
                             d->boundary_function > TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "boundary_function %d", d->boundary_function);
  if (d->nboundaries > 0 && d->boundary_function == TRIXI_IC_WEAK_BLAST_WAVE && d->equation == TRIXI_EQ_LINEAR_ADVECTION)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "the weak blast wave needs the Euler or MHD equations");
  if (d->nboundaries > 0 && d->boundary_function == TRIXI_IC_EOC_TEST_COUPLED_EULER_GRAVITY &&
      d->equation != TRIXI_EQ_COMPRESSIBLE_EULER)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "the Euler-gravity convergence test needs the Euler equations");
  if (d->nboundary_params < 0 || d->nboundary_params > 8 || d->nsource_params < 0 || d->nsource_params > 3)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "nboundary_params %d / nsource_params %d", d->nboundary_params,
                d->nsource_params);
  if (d->source_terms != TRIXI_SOURCE_NONE && d->source_terms != TRIXI_SOURCE_CONVERGENCE_TEST &&
      d->source_terms != TRIXI_SOURCE_EOC_TEST_EULER)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "source_terms %d", d->source_terms);
  if (d->source_terms != TRIXI_SOURCE_NONE && d->equation != TRIXI_EQ_COMPRESSIBLE_EULER)
    return fail(nullptr, TRIXI_ERR_UNSUPPORTED, "source terms %d are defined for the Euler equations", d->source_terms);
  if ((d->nboundaries > 0 || d->source_terms != TRIXI_SOURCE_NONE) && !d->node_coordinates)
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "boundaries and source terms need node_coordinates");
  if (d->nmortars < 0 || (d->nmortars > 0 && (!d->mortar_neighbor_ids || !d->mortar_large_sides || !d->mortar_orientations)))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "mortar tables");
  if (d->nmortars > 0 && d->ndims == 1) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "mortars in 1D");
  if (d->equation != TRIXI_EQ_LINEAR_ADVECTION && !(d->gamma > 1.0))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "gamma %g", d->gamma);

  trixi_handle *h = new trixi_handle();
  h->dim = d->ndims;
  h->N = d->polydeg + 1;
  h->nv = d->nvars;
  h->NF = (int)ipow64(h->N, h->dim - 1);
  h->NN = h->NF * h->N;
  h->nchild = 1 << (h->dim - 1);
  h->eq = d->equation == TRIXI_EQ_LINEAR_ADVECTION ? EQ_ADV : mhd ? EQ_MHD : EQ_EULER;
  h->c_h = d->glm_speed;
  h->vol = d->volume_integral;
  h->vflux = d->volume_flux;
  h->sflux = d->surface_flux;
  h->fvflux = d->volume_flux_fv;
  // the entropy-conservative flux of linear advection is the central flux
  if (h->eq == EQ_ADV && h->vflux == TRIXI_FLUX_RANOCHA) h->vflux = TRIXI_FLUX_CENTRAL;
  h->mixed = d->precision == TRIXI_PRECISION_MIXED;
  h->gamma = d->gamma;
  for (int i = 0; i < 3; ++i) h->adv[i] = d->advection_velocity[i];
  h->alpha_max = d->alpha_max;
  h->alpha_min = d->alpha_min;
  h->alpha_smooth = d->alpha_smooth;
  h->ind_var = d->volume_integral == TRIXI_VOLUME_SHOCK_CAPTURING_HG ? d->indicator_variable : 0;
  h->E = d->nelements;
  h->I = d->ninterfaces;
  h->M = d->nmortars;
  h->B = d->nboundaries;
  h->src_kind = d->source_terms;
  for (int i = 0; i < d->nsource_params; ++i) h->src[i] = d->source_params[i];
  if (!fused_supported(h->dim, h->N, h->eq, h->vol, h->vflux)) {
    int st = fail(nullptr, TRIXI_ERR_UNSUPPORTED, "volume integral %d with volume flux %d for equation %d",
                  h->vol, h->vflux, h->eq);
    delete h;
    return st;
  }
  if (!compute_basis(d->polydeg, h->basis)) {
    delete h;
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "basis for polydeg %d", d->polydeg);
  }
  {  // optional overrides with the caller's (e.g. Trixi.jl's) operators
    const size_t nn = (size_t)h->N * h->N;
    auto take = [&](const double *src, std::vector<double> &dst, size_t n) {
      if (src) dst.assign(src, src + n);
    };
    take(d->weights, h->basis.weights, h->N);
    take(d->derivative_split, h->basis.dsplit, nn);
    take(d->derivative_dhat, h->basis.dhat, nn);
    take(d->inverse_vandermonde_legendre, h->basis.ivdm, nn);
    take(d->forward_upper, h->basis.fwd_up, nn);
    take(d->forward_lower, h->basis.fwd_lo, nn);
    take(d->reverse_upper, h->basis.rev_up, nn);
    take(d->reverse_lower, h->basis.rev_lo, nn);
  }

  // face table: one entry per element face (direction 2*(o-1) = -o face,
  // 2*(o-1)+1 = +o face, the surface_flux_values direction order)
  const int nfaces = 2 * h->dim;
  const int nc = h->nchild;
  std::vector<int32_t> ft((size_t)h->E * nfaces, INT32_MIN);
  std::vector<int32_t> slot_nbrs((size_t)std::max<int64_t>(1, h->M * (nc + 1)) * 4, -1);
  auto bad = [&](const char *fmt, long long a, long long b) {
    int st = fail(nullptr, TRIXI_ERR_BAD_CONNECTIVITY, fmt, a, b);
    delete h;
    return st;
  };
  for (int64_t k = 0; k < h->I; ++k) {
    const int64_t l = d->interface_neighbor_ids[2 * k], r = d->interface_neighbor_ids[2 * k + 1];
    const int64_t o = d->interface_orientations[k];
    if (l < 1 || l > h->E || r < 1 || r > h->E) return bad("interface %lld: neighbour id out of range (%lld)", (long long)k + 1, (long long)(l < 1 || l > h->E ? l : r));
    if (o < 1 || o > h->dim) return bad("interface %lld: orientation %lld", (long long)k + 1, (long long)o);
    int32_t &fl = ft[(size_t)(l - 1) * nfaces + 2 * (o - 1) + 1];
    int32_t &fr = ft[(size_t)(r - 1) * nfaces + 2 * (o - 1)];
    if (fl != INT32_MIN || fr != INT32_MIN) return bad("interface %lld: face already connected (orientation %lld)", (long long)k + 1, (long long)o);
    fl = (int32_t)(r - 1);
    fr = (int32_t)(l - 1);
  }
  for (int64_t m = 0; m < h->M; ++m) {
    const int64_t o = d->mortar_orientations[m], ls = d->mortar_large_sides[m];
    if (o < 1 || o > h->dim) return bad("mortar %lld: orientation %lld", (long long)m + 1, (long long)o);
    if (ls != 1 && ls != 2) return bad("mortar %lld: large side %lld", (long long)m + 1, (long long)ls);
    const int small_dir = (int)(2 * (o - 1) + (ls - 1));
    const int large_dir = (int)(2 * (o - 1) + (ls == 1 ? 1 : 0));
    const int64_t large = d->mortar_neighbor_ids[nc + (nc + 1) * m];
    if (large < 1 || large > h->E) return bad("mortar %lld: large id %lld", (long long)m + 1, (long long)large);
    const int64_t base = m * (nc + 1);
    for (int c = 0; c < nc; ++c) {
      const int64_t s = d->mortar_neighbor_ids[c + (nc + 1) * m];
      if (s < 1 || s > h->E) return bad("mortar %lld: small id %lld", (long long)m + 1, (long long)s);
      int32_t &f = ft[(size_t)(s - 1) * nfaces + small_dir];
      if (f != INT32_MIN) return bad("mortar %lld: small face already connected (element %lld)", (long long)m + 1, (long long)s);
      f = (int32_t)(-(base + c) - 1);
      slot_nbrs[(size_t)(base + c) * 4] = (int32_t)(large - 1);
      slot_nbrs[(size_t)(base + nc) * 4 + c] = (int32_t)(s - 1);
    }
    int32_t &f = ft[(size_t)(large - 1) * nfaces + large_dir];
    if (f != INT32_MIN) return bad("mortar %lld: large face already connected (element %lld)", (long long)m + 1, (long long)large);
    f = (int32_t)(-(base + nc) - 1);
  }
  // boundary faces keep the FACE_BOUNDARY (= INT32_MIN) entry, once declared
  std::vector<char> declared(ft.size(), 0);
  for (int64_t b = 0; b < h->B; ++b) {
    const int64_t e = d->boundary_neighbor_ids[b], side = d->boundary_neighbor_sides[b], o = d->boundary_orientations[b];
    if (e < 1 || e > h->E) return bad("boundary %lld: element id %lld", (long long)b + 1, (long long)e);
    if (side != 1 && side != 2) return bad("boundary %lld: side %lld", (long long)b + 1, (long long)side);
    if (o < 1 || o > h->dim) return bad("boundary %lld: orientation %lld", (long long)b + 1, (long long)o);
    const size_t fi = (size_t)(e - 1) * nfaces + 2 * (o - 1) + (side == 1 ? 1 : 0);
    if (ft[fi] != INT32_MIN || declared[fi]) return bad("boundary %lld: face already connected (element %lld)", (long long)b + 1, (long long)e);
    declared[fi] = 1;
  }
  if (d->nghost_elements < 0 || d->nghost_elements >= h->E) return bad("nghost_elements %lld of %lld", (long long)d->nghost_elements, (long long)h->E);
  const int64_t first_ghost = h->E - d->nghost_elements;
  for (size_t i = 0; i < ft.size(); ++i)
    if (ft[i] == INT32_MIN && !declared[i]) {
      const int64_t e = (int64_t)(i / nfaces);
      if (e >= first_ghost) {
        ft[i] = (int32_t)e;  // open ghost face: read the ghost itself (its rhs is discarded)
        continue;
      }
      return bad("element %lld face %lld has no interface, mortar or boundary",
                 (long long)(i / nfaces) + 1, (long long)(i % nfaces) + 1);
    }

  for (int64_t e = 0; e < h->E; ++e) h->total_volume += std::pow(2.0 / d->inverse_jacobian[e], h->dim);
  // all host-side validation is done; from here on the device is touched
  cudaGetDevice(&h->device);
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  ok(upload(&h->d_face_table, ft.data(), ft.size()));
  ok(upload(&h->d_slot_nbrs, slot_nbrs.data(), slot_nbrs.size()));
  ok(upload(&h->d_inv_jac, d->inverse_jacobian, (size_t)h->E));
  ok(upload(&h->d_if_nid, d->interface_neighbor_ids, (size_t)(2 * h->I)));
  ok(upload(&h->d_if_ori, d->interface_orientations, (size_t)h->I));
  ok(upload(&h->d_mo_nid, d->mortar_neighbor_ids, (size_t)((nc + 1) * h->M)));
  ok(upload(&h->d_mo_ls, d->mortar_large_sides, (size_t)h->M));
  ok(upload(&h->d_mo_ori, d->mortar_orientations, (size_t)h->M));
  if (h->M > 0) ok(cudaMalloc(&h->d_mortar_flux, sizeof(double) * (size_t)(h->M * (nc + 1) * h->NF * h->nv)));
  if (h->vol == TRIXI_VOLUME_SHOCK_CAPTURING_HG) {
    ok(cudaMalloc(&h->d_alpha_raw, sizeof(double) * (size_t)h->E));
    ok(cudaMalloc(&h->d_alpha, sizeof(double) * (size_t)h->E));
    if (h->d_alpha) ok(cudaMemset(h->d_alpha, 0, sizeof(double) * (size_t)h->E));
  }
  if (d->node_coordinates)
    ok(upload(&h->d_coords, d->node_coordinates, (size_t)(h->dim * h->NN * h->E)));
  if (h->B > 0) {
    ok(upload(&h->d_bnd_nid, d->boundary_neighbor_ids, (size_t)h->B));
    ok(upload(&h->d_bnd_side, d->boundary_neighbor_sides, (size_t)h->B));
    ok(upload(&h->d_bnd_ori, d->boundary_orientations, (size_t)h->B));
  }
  ok(upload(&h->d_w, h->basis.weights.data(), (size_t)h->N));
  ok(cudaMalloc(&h->d_err, sizeof(int)));
  if (h->d_err) ok(cudaMemset(h->d_err, 0, sizeof(int)));
  if (e != cudaSuccess) {
    int st = cuda_fail(nullptr, e, "trixi_create");
    free_all(h);
    delete h;
    return st;
  }

  // fused-kernel launch template
  FusedHost &f = h->fused;
  f.face_table = h->d_face_table;
  f.mortar_flux = h->d_mortar_flux;
  f.inv_jac = h->d_inv_jac;
  f.alpha = h->d_alpha;
  f.err = h->d_err;
  f.nelements = h->E;
  f.surface_flux = h->sflux;
  f.fv_flux = h->fvflux;
  const double eps = 2.220446049250313e-16;
  f.atol = std::max(100 * eps, std::pow(eps, 0.75));  // src/solvers/dg_2d.jl:173
  f.gamma = h->gamma;
  for (int i = 0; i < 3; ++i) f.adv[i] = h->adv[i];
  f.c_h = h->c_h;
  f.N = h->N;
  to_row_major(h->basis.dsplit, h->N, f.dsplit);
  for (int i = 0; i < h->N; ++i) f.dsplit[i * h->N + i] = 0.0;  // zeroed diagonal (dg_2d_kernel.jl:189-190)
  to_row_major(h->basis.dhat, h->N, f.dhat);
  for (int i = 0; i < h->N; ++i) f.invw[i] = 1.0 / h->basis.weights[i];
  f.lhat_l = 1.0 / h->basis.weights[0];          // boundary_interpolation[1, 1]
  f.lhat_r = 1.0 / h->basis.weights[h->N - 1];   // boundary_interpolation[N, 2]
  h->bc_kind = h->B > 0 ? d->boundary_function : -1;
  h->bc = ic_params(h, h->bc_kind, d->boundary_params, d->nboundary_params);
  f.coords = h->d_coords;
  f.pdl = 1;  // programmatic dependent launches: stage s+1 overlaps its launch with stage s's last wave
  f.bc_kind = h->bc_kind;
  f.bc = h->bc;
  f.src_kind = h->src_kind;
  for (int i = 0; i < 3; ++i) f.src[i] = h->src[i];
  *out = h;
  return TRIXI_OK;
}

int trixi_destroy(trixi_handle *h) {
  if (!h) return TRIXI_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != h->device) cudaSetDevice(h->device);
  free_all(h);
  if (cur != h->device) cudaSetDevice(cur);
  delete h;
  return TRIXI_OK;
}

}  // extern "C"

namespace {

void fill_mortar(const trixi_handle *h, MortarHost &mh, const double *u) {
  mh.dim = h->dim;
  mh.N = h->N;
  mh.eq = h->eq;
  mh.nv = h->nv;
  mh.nmortars = h->M;
  mh.u = u;
  mh.neighbor_ids = h->d_mo_nid;
  mh.large_sides = h->d_mo_ls;
  mh.orientations = h->d_mo_ori;
  mh.mortar_flux = h->d_mortar_flux;
  mh.surface_flux = h->sflux;
  mh.mixed = h->mixed;
  mh.gamma = h->gamma;
  mh.c_h = h->c_h;
  for (int i = 0; i < 3; ++i) mh.adv[i] = h->adv[i];
  to_row_major(h->basis.fwd_up, h->N, mh.fwd_up);
  to_row_major(h->basis.fwd_lo, h->N, mh.fwd_lo);
  to_row_major(h->basis.rev_up, h->N, mh.rev_up);
  to_row_major(h->basis.rev_lo, h->N, mh.rev_lo);
  mh.err = h->d_err;
}

// fp32: the indicator inside an FP32-mixed rhs; the stage entry point
// trixi_indicator always computes in FP64
int run_indicator(trixi_handle *h, const double *u, double *alpha_out, cudaStream_t s, bool fp32 = false,
                  const float *u32 = nullptr) {
  IndicatorHost ih;
  ih.dim = h->dim;
  ih.N = h->N;
  ih.nv = h->nv;
  ih.eq = h->eq;
  ih.mixed = fp32;
  ih.variable = h->ind_var;
  ih.nelements = h->E;
  ih.u = u;
  ih.u32 = fp32 ? u32 : nullptr;
  ih.pdl = h->fused.pdl;  // chained with the fused kernels as programmatic dependent launches
  ih.alpha_raw = h->d_alpha_raw;
  ih.alpha = alpha_out;
  ih.face_table = h->d_face_table;
  ih.slot_neighbors = h->d_slot_nbrs;
  ih.smooth = h->alpha_smooth;
  ih.gamma = h->gamma;
  ih.alpha_max = h->alpha_max;
  ih.alpha_min = h->alpha_min;
  // src/solvers/indicators.jl:22-24
  ih.threshold = 0.5 * std::pow(10.0, -1.8 * std::pow((double)h->N, 0.25));
  ih.parameter_s = std::log((1 - 0.0001) / 0.0001);
  to_row_major(h->basis.ivdm, h->N, ih.ivdm);
  TRIXI_CUDA(h, launch_indicator(ih, s), "indicator");
  return TRIXI_OK;
}

// Kernels of one rhs evaluation (mode RHS/RK/VOLUME) on u_in.  u32_in /
// u32_out: FP32 copies of u_in / out for FP32-mixed RK stages (or null).
int run_rhs(trixi_handle *h, int mode, const double *u_in, double *out, double *k, double a, double b, double dt,
            cudaStream_t s, double t = 0.0, const float *u32_in = nullptr, float *u32_out = nullptr) {
  if (h->vol == TRIXI_VOLUME_SHOCK_CAPTURING_HG) {
    int st = run_indicator(h, u_in, h->d_alpha, s, h->mixed && mode != MODE_VOLUME, u32_in);
    if (st) return st;
  }
  if (h->M > 0 && mode != MODE_VOLUME) {
    MortarHost mh;
    fill_mortar(h, mh, u_in);
    TRIXI_CUDA(h, launch_mortar_flux(mh, s), "mortar flux");
  }
  FusedHost f = h->fused;
  f.u_in = u_in;
  f.out = out;
  f.k = k;
  f.mode = mode;
  f.rk_a = a;
  f.rk_b = b;
  f.dt = dt;
  f.t = t;
  f.u32_in = u32_in;
  f.u32_out = u32_out;
  TRIXI_CUDA(h, launch_fused(h->dim, h->N, h->eq, h->vol, h->vflux, h->mixed, f, s), "fused rhs");
  return TRIXI_OK;
}

int fused_tile(trixi_handle *h, FusedTile &t) {
  FusedHost f = h->fused;
  f.tile_out = &t;
  f.nelements = 0;
  TRIXI_CUDA(h, launch_fused(h->dim, h->N, h->eq, h->vol, h->vflux, h->mixed, f, nullptr), "fused tile query");
  return TRIXI_OK;
}

// Tile tuner: times the fused RK-stage launch for every valid (warps per
// group, groups per block) on the state u (read only; the outputs go to
// temporary buffers) and keeps the fastest.  Results do not depend on the
// tile: every node and flux is computed by the same arithmetic.
int tune_tiles(trixi_handle *h, const double *u, cudaStream_t s) {
  FusedTile t;
  if (int st = fused_tile(h, t)) return st;
  struct Cand {
    int w, g;
  };
  std::vector<Cand> cand;
  for (int w = t.min_wpg; w <= 8; ++w)
    for (int g : {1, 2, 4, 8})
      if (g * w <= t.max_warps && (size_t)g * t.group_smem <= 200 * 1024) cand.push_back({w, g});
  const size_t bytes = sizeof(double) * (size_t)(h->E * h->NN * h->nv);
  double *out = nullptr, *k = nullptr;
  TRIXI_CUDA(h, cudaMalloc(&out, bytes), "tuner buffers");
  if (cudaMalloc(&k, bytes) != cudaSuccess) {
    cudaFree(out);
    return fail(h, TRIXI_ERR_OUT_OF_MEMORY, "tuner buffers");
  }
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  int status = TRIXI_OK;
  h->tune_wpg.clear();
  h->tune_gpb.clear();
  h->tune_ms.clear();
  const FusedHost saved = h->fused;
  int best_w = 0, best_g = 0;
  double best_ms = 0.0;
  if (cudaMemsetAsync(k, 0, bytes, s) != cudaSuccess) status = fail(h, TRIXI_ERR_CUDA, "tuner k");
  for (size_t ci = 0; ci < cand.size() && status == TRIXI_OK; ++ci) {
    h->fused.wpg = cand[ci].w;
    h->fused.gpb = cand[ci].g;
    const int reps = 5;
    status = run_rhs(h, MODE_RK, u, out, k, 0.5, 0.1, 1e-9, s);  // warm-up
    cudaEventRecord(t0, s);
    for (int r = 0; r < reps && status == TRIXI_OK; ++r) status = run_rhs(h, MODE_RK, u, out, k, 0.5, 0.1, 1e-9, s);
    cudaEventRecord(t1, s);
    if (status != TRIXI_OK) break;
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(t1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (e != cudaSuccess) {
      status = fail(h, TRIXI_ERR_CUDA, "tuner timing: %s", cudaGetErrorString(e));
      break;
    }
    h->tune_wpg.push_back(cand[ci].w);
    h->tune_gpb.push_back(cand[ci].g);
    h->tune_ms.push_back(ms / reps);
    if (best_w == 0 || ms / reps < best_ms) {
      best_w = cand[ci].w;
      best_g = cand[ci].g;
      best_ms = ms / reps;
    }
  }
  cudaStreamSynchronize(s);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  cudaFree(k);
  h->fused = saved;
  if (status != TRIXI_OK) return status;
  h->fused.wpg = best_w;
  h->fused.gpb = best_g;
  return TRIXI_OK;
}

StageHost stage_of(trixi_handle *h) {
  StageHost sh;
  sh.dim = h->dim;
  sh.N = h->N;
  sh.nv = h->nv;
  sh.eq = h->eq;
  sh.nelements = h->E;
  sh.ninterfaces = h->I;
  sh.nmortars = h->M;
  sh.if_neighbor_ids = h->d_if_nid;
  sh.if_orientations = h->d_if_ori;
  sh.mo_neighbor_ids = h->d_mo_nid;
  sh.mo_large_sides = h->d_mo_ls;
  sh.mo_orientations = h->d_mo_ori;
  sh.interfaces_u = h->d_interfaces_u;
  sh.sfv = h->d_sfv;
  for (int c = 0; c < 4; ++c) sh.mortar_u[c] = h->d_mortar_u[c];
  sh.surface_flux = h->sflux;
  sh.gamma = h->gamma;
  sh.c_h = h->c_h;
  for (int i = 0; i < 3; ++i) sh.adv[i] = h->adv[i];
  to_row_major(h->basis.fwd_up, h->N, sh.fwd_up);
  to_row_major(h->basis.fwd_lo, h->N, sh.fwd_lo);
  to_row_major(h->basis.rev_up, h->N, sh.rev_up);
  to_row_major(h->basis.rev_lo, h->N, sh.rev_lo);
  sh.lhat_l = 1.0 / h->basis.weights[0];
  sh.lhat_r = 1.0 / h->basis.weights[h->N - 1];
  sh.inv_jac = h->d_inv_jac;
  sh.nboundaries = h->B;
  sh.bnd_neighbor_ids = h->d_bnd_nid;
  sh.bnd_sides = h->d_bnd_side;
  sh.bnd_orientations = h->d_bnd_ori;
  sh.boundaries_u = h->d_boundaries_u;
  sh.coords = h->d_coords;
  sh.bc_kind = h->bc_kind;
  sh.bc = h->bc;
  sh.src_kind = h->src_kind;
  for (int i = 0; i < 3; ++i) sh.src[i] = h->src[i];
  return sh;
}

// Stage containers are created on first use and then reused.
int ensure_stage_containers(trixi_handle *h) {
  if (h->d_sfv) return TRIXI_OK;
  const size_t iu = (size_t)std::max<int64_t>(1, 2 * h->nv * h->NF * h->I);
  const size_t sfv = (size_t)(h->nv * h->NF * 2 * h->dim * h->E);
  TRIXI_CUDA(h, cudaMalloc(&h->d_interfaces_u, sizeof(double) * iu), "alloc interfaces_u");
  TRIXI_CUDA(h, cudaMemset(h->d_interfaces_u, 0, sizeof(double) * iu), "init interfaces_u");
  TRIXI_CUDA(h, cudaMalloc(&h->d_sfv, sizeof(double) * sfv), "alloc surface_flux_values");
  TRIXI_CUDA(h, cudaMemset(h->d_sfv, 0, sizeof(double) * sfv), "init surface_flux_values");
  if (h->M > 0)
    for (int c = 0; c < h->nchild; ++c) {
      const size_t n = (size_t)(2 * h->nv * h->NF * h->M);
      TRIXI_CUDA(h, cudaMalloc(&h->d_mortar_u[c], sizeof(double) * n), "alloc mortar u");
      TRIXI_CUDA(h, cudaMemset(h->d_mortar_u[c], 0, sizeof(double) * n), "init mortar u");
    }
  if (h->B > 0) {
    const size_t n = (size_t)(2 * h->nv * h->NF * h->B);
    TRIXI_CUDA(h, cudaMalloc(&h->d_boundaries_u, sizeof(double) * n), "alloc boundaries u");
    TRIXI_CUDA(h, cudaMemset(h->d_boundaries_u, 0, sizeof(double) * n), "init boundaries u");
  }
  return TRIXI_OK;
}

}  // namespace

extern "C" {

int trixi_rhs(trixi_handle *h, double *du, const double *u, double t, void *stream) {
  (void)t;  // autonomous: no source terms, periodic boundaries
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, du, "du")) return st;
  if (int st = check_u_args(h, u, "u")) return st;
  if ((const void *)du == (const void *)u) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "du aliases u");
  return run_rhs(h, MODE_RHS, u, du, nullptr, 0, 0, 0, (cudaStream_t)stream, t);
}

int trixi_rk_stage(trixi_handle *h, double *u_out, const double *u_in, double *k, double a, double b, double dt,
                   double t, void *stream) {
  (void)t;
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u_out, "u_out")) return st;
  if (int st = check_u_args(h, u_in, "u_in")) return st;
  if (int st = check_u_args(h, k, "k")) return st;
  if ((const void *)u_out == (const void *)u_in) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "u_out aliases u_in");
  if (!std::isfinite(a) || !std::isfinite(b) || !std::isfinite(dt))
    return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "non-finite RK coefficient");
  return run_rhs(h, MODE_RK, u_in, u_out, k, a, b, dt, (cudaStream_t)stream, t);
}

int trixi_rk_steps(trixi_handle *h, double *u, double *k, double t, double dt, int64_t nsteps, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_u_args(h, k, "k")) return st;
  if (nsteps < 0 || !std::isfinite(dt)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "nsteps %lld / dt", (long long)nsteps);
  if (nsteps == 0) return TRIXI_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = sizeof(double) * (size_t)(h->E * h->NN * h->nv);
  if (!h->d_scratch_u) TRIXI_CUDA(h, cudaMalloc(&h->d_scratch_u, bytes), "alloc RK scratch");
  if (!h->d_scratch_u2) TRIXI_CUDA(h, cudaMalloc(&h->d_scratch_u2, bytes), "alloc RK scratch");
  // FP32-mixed Euler / MHD: each stage also writes its output narrowed to
  // FP32, and the next stage reads its flux states (and the shock indicator
  // its input) from that copy instead of narrowing the FP64 state again; the
  // results are the same bits.  The first stage of a call narrows the
  // caller's u, which may have changed since the previous call.
  const bool copies = h->mixed && h->eq != EQ_ADV;
  if (copies && !h->d_u32[0]) {
    const size_t fbytes = sizeof(float) * (size_t)(h->E * h->NN * h->nv);
    TRIXI_CUDA(h, cudaMalloc(&h->d_u32[0], fbytes), "alloc FP32 stage copy");
    TRIXI_CUDA(h, cudaMalloc(&h->d_u32[1], fbytes), "alloc FP32 stage copy");
  }
  // the stage inputs and outputs of one step: u -> s1 -> s2 -> s1 -> s2 -> u, so
  // that every step ends in the caller's buffer (u_out never aliases u_in)
  double *const seq[6] = {u, h->d_scratch_u, h->d_scratch_u2, h->d_scratch_u, h->d_scratch_u2, u};
  const int64_t nstages = 5 * nsteps;
  int64_t g = 0;  // stage counter of this call
  for (int64_t step = 0; step < nsteps; ++step) {
    for (int st = 0; st < 5; ++st, ++g) {
      const float *c_in = (copies && g > 0) ? h->d_u32[g & 1] : nullptr;
      float *c_out = (copies && g + 1 < nstages) ? h->d_u32[(g + 1) & 1] : nullptr;
      int r = run_rhs(h, MODE_RK, seq[st], seq[st + 1], k, kCK_A[st], kCK_B[st], dt, s, t + kCK_C[st] * dt, c_in,
                      c_out);
      if (r) return r;
    }
    t += dt;
  }
  return TRIXI_OK;
}

int trixi_rk_steps_host(trixi_handle *h, const double *u_in, double *u_out, double t, double dt, int64_t nsteps,
                        void *wait_event, void *done_event, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (!u_in || !u_out) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "host state pointer is null");
  if (nsteps < 0 || !std::isfinite(dt)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "nsteps %lld / dt", (long long)nsteps);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = sizeof(double) * (size_t)(h->E * h->NN * h->nv);
  if (!h->d_host_u) TRIXI_CUDA(h, cudaMalloc(&h->d_host_u, bytes), "alloc host-path state");
  if (!h->d_host_k) TRIXI_CUDA(h, cudaMalloc(&h->d_host_k, bytes), "alloc host-path register");
  TRIXI_CUDA(h, cudaMemcpyAsync(h->d_host_u, u_in, bytes, cudaMemcpyHostToDevice, s), "upload u");
  if (wait_event) TRIXI_CUDA(h, cudaStreamWaitEvent(s, (cudaEvent_t)wait_event, 0), "wait_event");
  if (int r = trixi_rk_steps(h, h->d_host_u, h->d_host_k, t, dt, nsteps, stream)) return r;
  if (done_event) TRIXI_CUDA(h, cudaEventRecord((cudaEvent_t)done_event, s), "done_event");
  TRIXI_CUDA(h, cudaMemcpyAsync(u_out, h->d_host_u, bytes, cudaMemcpyDeviceToHost, s), "download u");
  return TRIXI_OK;
}

int trixi_volume_integral(trixi_handle *h, double *du, const double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, du, "du")) return st;
  if (int st = check_u_args(h, u, "u")) return st;
  return run_rhs(h, MODE_VOLUME, u, du, nullptr, 0, 0, 0, (cudaStream_t)stream);
}

int trixi_prolong2interfaces(trixi_handle *h, const double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_prolong2interfaces(stage_of(h), u, (cudaStream_t)stream), "prolong2interfaces");
  return TRIXI_OK;
}

int trixi_interface_flux(trixi_handle *h, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_interface_flux(stage_of(h), (cudaStream_t)stream), "interface_flux");
  return TRIXI_OK;
}

int trixi_prolong2boundaries(trixi_handle *h, const double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (h->B == 0) return TRIXI_OK;  // periodic TreeMesh: no boundaries (src/solvers/dg_2d.jl:419-422)
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_prolong2boundaries(stage_of(h), u, (cudaStream_t)stream), "prolong2boundaries");
  return TRIXI_OK;
}

int trixi_boundary_flux(trixi_handle *h, double t, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (h->B == 0) return TRIXI_OK;  // periodic TreeMesh: no boundaries (src/solvers/dg_2d.jl:447-450)
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_boundary_flux(stage_of(h), t, (cudaStream_t)stream), "boundary_flux");
  return TRIXI_OK;
}

int trixi_prolong2mortars(trixi_handle *h, const double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_prolong2mortars(stage_of(h), u, (cudaStream_t)stream), "prolong2mortars");
  return TRIXI_OK;
}

int trixi_mortar_flux(trixi_handle *h, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_mortar_flux(stage_of(h), (cudaStream_t)stream), "mortar_flux");
  return TRIXI_OK;
}

int trixi_surface_integral(trixi_handle *h, double *du, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, du, "du")) return st;
  if (int st = ensure_stage_containers(h)) return st;
  TRIXI_CUDA(h, stage_surface_integral(stage_of(h), du, (cudaStream_t)stream), "surface_integral");
  return TRIXI_OK;
}

int trixi_jacobian(trixi_handle *h, double *du, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, du, "du")) return st;
  TRIXI_CUDA(h, stage_jacobian(stage_of(h), du, (cudaStream_t)stream), "jacobian");
  return TRIXI_OK;
}

int trixi_sources(trixi_handle *h, double *du, const double *u, double t, void *stream) {
  (void)u;  // the convergence-test source depends on (x, t) only
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (h->src_kind == 0) return TRIXI_OK;  // source_terms = nothing (src/solvers/dg_2d.jl:741-743)
  if (int st = check_u_args(h, du, "du")) return st;
  TRIXI_CUDA(h, stage_sources(stage_of(h), du, t, (cudaStream_t)stream), "sources");
  return TRIXI_OK;
}

int trixi_container(trixi_handle *h, int which, void **dev_ptr, int64_t *count) {
  if (!h || !dev_ptr || !count) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "null argument");
  if (which == TRIXI_CONTAINER_ALPHA) {
    *dev_ptr = h->d_alpha;
    *count = h->d_alpha ? h->E : 0;
    return TRIXI_OK;
  }
  if (which == TRIXI_CONTAINER_INVERSE_JACOBIAN) {
    *dev_ptr = h->d_inv_jac;
    *count = h->E;
    return TRIXI_OK;
  }
  if (int st = ensure_stage_containers(h)) return st;
  if (which == TRIXI_CONTAINER_INTERFACES_U) {
    *dev_ptr = h->d_interfaces_u;
    *count = 2 * h->nv * h->NF * h->I;
    return TRIXI_OK;
  }
  if (which == TRIXI_CONTAINER_BOUNDARIES_U) {
    *dev_ptr = h->d_boundaries_u;
    *count = 2 * h->nv * h->NF * h->B;
    return TRIXI_OK;
  }
  if (which == TRIXI_CONTAINER_SURFACE_FLUX_VALUES) {
    *dev_ptr = h->d_sfv;
    *count = h->nv * h->NF * 2 * h->dim * h->E;
    return TRIXI_OK;
  }
  if (which >= TRIXI_CONTAINER_MORTARS_U && which < TRIXI_CONTAINER_MORTARS_U + h->nchild && h->dim > 1) {
    // reference order: 2D u_upper, u_lower; 3D u_upper_left, u_upper_right, u_lower_left, u_lower_right
    static const int map2[2] = {1, 0};
    static const int map3[4] = {2, 3, 0, 1};
    const int j = which - TRIXI_CONTAINER_MORTARS_U;
    const int c = (h->dim == 2) ? map2[j] : map3[j];
    *dev_ptr = h->d_mortar_u[c];
    *count = h->M > 0 ? 2 * h->nv * h->NF * h->M : 0;
    return TRIXI_OK;
  }
  return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "container %d", which);
}

int trixi_indicator(trixi_handle *h, const double *u, double *alpha, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (h->eq == EQ_ADV) return fail(h, TRIXI_ERR_UNSUPPORTED, "indicator on density_pressure needs Euler or MHD");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_u_args(h, alpha, "alpha")) return st;
  if (!h->d_alpha_raw) {
    TRIXI_CUDA(h, cudaMalloc(&h->d_alpha_raw, sizeof(double) * (size_t)h->E), "alloc alpha");
  }
  return run_indicator(h, u, alpha, (cudaStream_t)stream);
}

static int copy_basis_item(const Basis &b, int which, double *host_out, int64_t count) {
  if (!host_out) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "null argument");
  const std::vector<double> *src = nullptr;
  switch (which) {
    case 0: src = &b.nodes; break;
    case 1: src = &b.weights; break;
    case 2: src = &b.dsplit; break;
    case 3: src = &b.dhat; break;
    case 4: src = &b.ivdm; break;
    case 5: src = &b.fwd_up; break;
    case 6: src = &b.fwd_lo; break;
    case 7: src = &b.rev_up; break;
    case 8: src = &b.rev_lo; break;
    case 9: src = &b.dmat; break;
    default: return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "basis item %d", which);
  }
  if (count < (int64_t)src->size())
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "count %lld < %lld", (long long)count, (long long)src->size());
  std::memcpy(host_out, src->data(), sizeof(double) * src->size());
  return TRIXI_OK;
}

int trixi_basis(const trixi_handle *h, int which, double *host_out, int64_t count) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  return copy_basis_item(h->basis, which, host_out, count);
}

int trixi_lgl_basis(int polydeg, int which, double *host_out, int64_t count) {
  Basis b;
  if (polydeg < 1 || polydeg > 15 || !compute_basis(polydeg, b))
    return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "polydeg %d", polydeg);
  return copy_basis_item(b, which, host_out, count);
}

int trixi_autotune(trixi_handle *h, const double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (!aligned8(u)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "u must be an 8-byte aligned device pointer");
  if (h->E == 0) return TRIXI_OK;
  return tune_tiles(h, u, (cudaStream_t)stream);
}

int trixi_set_tile(trixi_handle *h, int wpg, int gpb) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (wpg == 0 && gpb == 0) {
    h->fused.wpg = h->fused.gpb = 0;
    return TRIXI_OK;
  }
  FusedTile t;
  if (int st = fused_tile(h, t)) return st;
  if (wpg < t.min_wpg || wpg > 8 || gpb < 1 || gpb > 15 || gpb * wpg > t.max_warps ||
      (size_t)gpb * t.group_smem > 200 * 1024)
    return fail(h, TRIXI_ERR_INVALID_ARGUMENT,
                "tile (%d warps per group, %d groups per block) outside [%d..8] warps, <= %d warps per block", wpg,
                gpb, t.min_wpg, t.max_warps);
  h->fused.wpg = wpg;
  h->fused.gpb = gpb;
  return TRIXI_OK;
}

int trixi_set_glm_speed(trixi_handle *h, double c_h) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (h->eq != EQ_MHD) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "the GLM speed belongs to ideal GLM-MHD");
  h->c_h = c_h;
  h->fused.c_h = c_h;
  return TRIXI_OK;
}

int trixi_tile(trixi_handle *h, int *epg, int *wpg, int *gpb, int *cand_wpg, int *cand_gpb, double *cand_ms,
               int64_t max, int64_t *count) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  FusedTile t;
  if (int st = fused_tile(h, t)) return st;
  const bool custom = h->fused.wpg > 0 && h->fused.gpb > 0;
  if (epg) *epg = t.epg;
  if (wpg) *wpg = custom ? h->fused.wpg : t.def_wpg;
  if (gpb) *gpb = custom ? h->fused.gpb : t.def_gpb;
  const int64_t n = (int64_t)h->tune_ms.size();
  if (count) *count = n;
  for (int64_t i = 0; i < n && i < max; ++i) {
    if (cand_wpg) cand_wpg[i] = h->tune_wpg[(size_t)i];
    if (cand_gpb) cand_gpb[i] = h->tune_gpb[(size_t)i];
    if (cand_ms) cand_ms[i] = h->tune_ms[(size_t)i];
  }
  return TRIXI_OK;
}

int trixi_synchronize(trixi_handle *h, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  TRIXI_CUDA(h, cudaStreamSynchronize((cudaStream_t)stream), "synchronize");
  int flag = 0;
  TRIXI_CUDA(h, cudaMemcpy(&flag, h->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read error word");
  if (flag) return fail(h, TRIXI_ERR_DEVICE_FLAG, "device error word %d", flag);
  return TRIXI_OK;
}

}  // extern "C"

namespace {

IcParams ic_params(const trixi_handle *h, int kind, const double *params, int64_t nparams) {
  IcParams ip{};
  for (int i = 0; i < 3; ++i) ip.a[i] = h->adv[i];
  ip.gamma = h->gamma;
  if (kind == IC_CONVERGENCE_TEST) {
    if (h->eq == EQ_ADV) {
      ip.p[0] = 1.0; ip.p[1] = 0.5; ip.p[2] = 2.0;
    } else {
      ip.p[0] = 2.0; ip.p[1] = 0.1; ip.p[2] = 2.0;
    }
  }
  for (int64_t i = 0; params && i < nparams && i < 9; ++i) ip.p[i] = params[i];
  for (size_t i = 0; i < h->xa.size() && i < 16; ++i) ip.xa[i] = h->xa[i];
  return ip;
}

int check_ic(trixi_handle *h, int kind, int64_t nparams, const double *params) {
  if (kind < IC_CONSTANT || kind > IC_LAST) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "ic kind %d", kind);
  if (kind == IC_WEAK_BLAST_WAVE && h->eq == EQ_ADV)
    return fail(h, TRIXI_ERR_UNSUPPORTED, "weak blast wave needs the Euler or MHD equations");
  if (kind == IC_EOC_EULER_GRAVITY && h->eq != EQ_EULER)
    return fail(h, TRIXI_ERR_UNSUPPORTED, "the Euler-gravity convergence test needs the Euler equations");
  if (kind == IC_CONSTANT && (!params || nparams < h->nv))
    return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "constant state needs %d params", h->nv);
  if (nparams < 0 || nparams > 9) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "nparams %lld", (long long)nparams);
  return TRIXI_OK;
}

// results of the single-block reductions: up to kRedSlot values (the nvars
// of one quantity, at most 9) from offset 0, and a second set (Linf) from
// offset kRedSlot
constexpr int kRedSlot = 16;
constexpr int kRedOut = 2 * kRedSlot;

int ensure_reduction(trixi_handle *h, int nq) {
  if (nq > kRedSlot || h->nv > kRedSlot) return fail(h, TRIXI_ERR_UNSUPPORTED, "reduction of %d values", nq);
  if (!h->d_acc) TRIXI_CUDA(h, cudaMalloc(&h->d_acc, sizeof(unsigned long long)), "alloc reduction");
  if (!h->d_partial) {
    // sized for the largest quantity any call asks for (nvars per element),
    // whichever call allocates first
    const size_t per = (size_t)std::max(h->nv, 5);
    TRIXI_CUDA(h, cudaMalloc(&h->d_partial, sizeof(double) * (size_t)h->E * per), "alloc partials");
    TRIXI_CUDA(h, cudaMalloc(&h->d_partial2, sizeof(double) * (size_t)h->E * per), "alloc partials");
    TRIXI_CUDA(h, cudaMalloc(&h->d_red_out, sizeof(double) * kRedOut), "alloc reduction out");
  }
  return TRIXI_OK;
}

}  // namespace

extern "C" {

int trixi_compute_coefficients(trixi_handle *h, int ic_kind, const double *params, int64_t nparams, double t,
                               double *u, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_ic(h, ic_kind, nparams, params)) return st;
  if (!h->d_coords) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "desc.node_coordinates was not given");
  IcHost ih;
  ih.dim = h->dim;
  ih.eq = h->eq;
  ih.N = h->N;
  ih.kind = ic_kind;
  ih.E = h->E;
  ih.coords = h->d_coords;
  ih.ip = ic_params(h, ic_kind, params, nparams);
  ih.t = t;
  ih.u = u;
  TRIXI_CUDA(h, launch_initial_condition(ih, (cudaStream_t)stream), "initial condition");
  return TRIXI_OK;
}

int trixi_max_dt(trixi_handle *h, const double *u, double *dt_dev, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_u_args(h, dt_dev, "dt")) return st;
  if (int st = ensure_reduction(h, 1)) return st;
  MaxDtHost mh;
  mh.dim = h->dim;
  mh.eq = h->eq;
  mh.N = h->N;
  mh.E = h->E;
  mh.u = u;
  mh.inv_jac = h->d_inv_jac;
  mh.gamma = h->gamma;
  for (int i = 0; i < 3; ++i) mh.a[i] = h->adv[i];
  mh.acc = h->d_acc;
  mh.dt = dt_dev;
  TRIXI_CUDA(h, launch_max_dt(mh, (cudaStream_t)stream), "max_dt");
  return TRIXI_OK;
}

int trixi_integrate(trixi_handle *h, const double *u, const double *du, int which, double *out_host, int64_t count,
                    void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (which < 0 || which > 3) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "integral kind %d", which);
  if ((which == 2 || which == 3) && !aligned8(du)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "du is required");
  const int nq = (which == 0 || which == 3) ? h->nv : 1;
  if (!out_host || count < nq) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "output needs %d values", nq);
  if (int st = ensure_reduction(h, nq)) return st;
  IntegrateHost ih;
  ih.dim = h->dim;
  ih.eq = h->eq;
  ih.N = h->N;
  ih.which = which;
  ih.nq = nq;
  ih.E = h->E;
  ih.u = u;
  ih.du = du;
  ih.inv_jac = h->d_inv_jac;
  ih.w = h->d_w;
  ih.gamma = h->gamma;
  ih.partial = h->d_partial;
  ih.out = h->d_red_out;
  cudaStream_t s = (cudaStream_t)stream;
  TRIXI_CUDA(h, launch_integrate(ih, s), "integrate");
  TRIXI_CUDA(h, cudaMemcpyAsync(out_host, h->d_red_out, sizeof(double) * nq, cudaMemcpyDeviceToHost, s), "copy");
  TRIXI_CUDA(h, cudaStreamSynchronize(s), "synchronize");
  return TRIXI_OK;
}

int trixi_calc_error_norms(trixi_handle *h, const double *u, const double *u_ref, int ic_kind, const double *params,
                           int64_t nparams, double t, double *l2_host, double *linf_host, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (!l2_host || !linf_host) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "null output");
  if (!u_ref) {
    if (int st = check_ic(h, ic_kind, nparams, params)) return st;
  } else if (!aligned8(u_ref)) {
    return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "u_ref misaligned");
  }
  if (!h->d_coords && !u_ref) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "desc.node_coordinates was not given");
  if (int st = ensure_reduction(h, h->nv)) return st;
  const int na = 2 * (h->N - 1) + 1;  // SolutionAnalyzer: analysis_polydeg = 2 polydeg
  if (!h->d_vdm) {
    std::vector<double> vdm, wa, xa;
    if (!analysis_operators(h->N - 1, na, vdm, wa, xa)) return fail(h, TRIXI_ERR_UNSUPPORTED, "analysis nodes");
    TRIXI_CUDA(h, upload(&h->d_vdm, vdm.data(), vdm.size()), "upload analysis operators");
    TRIXI_CUDA(h, upload(&h->d_wa, wa.data(), wa.size()), "upload analysis weights");
    h->xa = xa;
  }
  ErrorNormHost eh;
  eh.dim = h->dim;
  eh.eq = h->eq;
  eh.N = h->N;
  eh.NA = na;
  eh.nv = h->nv;
  eh.kind = ic_kind;
  eh.E = h->E;
  eh.u = u;
  eh.uref = u_ref;
  eh.coords = h->d_coords;
  eh.ip = ic_params(h, ic_kind, params, nparams);
  eh.t = t;
  eh.vdm = h->d_vdm;
  eh.wa = h->d_wa;
  eh.inv_jac = h->d_inv_jac;
  eh.l2p = h->d_partial;
  eh.linfp = h->d_partial2;
  eh.l2_out = h->d_red_out;
  eh.linf_out = h->d_red_out + kRedSlot;
  cudaStream_t s = (cudaStream_t)stream;
  if (!h->d_coords) {
    // coordinates are only read for the analytic reference; give a harmless pointer
    eh.coords = h->d_inv_jac;
  }
  TRIXI_CUDA(h, launch_error_norms_all(eh, s), "error norms");
  double buf[kRedOut];
  TRIXI_CUDA(h, cudaMemcpyAsync(buf, h->d_red_out, sizeof(double) * kRedOut, cudaMemcpyDeviceToHost, s), "copy");
  TRIXI_CUDA(h, cudaStreamSynchronize(s), "synchronize");
  // total volume = sum_e (2 / J^{-1}_e)^d: L2 is normalised by it
  double vol = 0.0;
  if (h->total_volume <= 0.0) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "total volume");
  vol = h->total_volume;
  for (int v = 0; v < h->nv; ++v) {
    l2_host[v] = std::sqrt(buf[v] / vol);
    linf_host[v] = buf[kRedSlot + v];
  }
  return TRIXI_OK;
}

}  // extern "C"

// ===========================================================================
// Batched ensembles: many independent instances advanced together.
//
// Instances with the same kernel kind (ndims, polydeg, equation, volume
// integral and fluxes) are merged into one group: their elements are
// concatenated and their connectivity offset, so that a group is one mesh
// with disconnected components and is served by a single fused launch per
// RK stage, whatever the number of instances in it.  Each element carries
// the time step of its instance.  A whole CarpenterKennedy2N54 step (all
// groups, all stages, mortar kernels included) is captured once as a CUDA
// graph and replayed.
// ===========================================================================

struct trixi_batch {
  struct Group {
    trixi_handle *h = nullptr;
    int64_t value_offset = 0;  // offset of the group's first value in the batch state
    int64_t nvalues = 0;
    std::vector<int64_t> instances;
    double *d_dt = nullptr;    // [group elements]
  };
  std::vector<Group> groups;
  std::vector<int64_t> inst_group, inst_offset, inst_nvalues, inst_nelem;
  int64_t total_values = 0;
  std::vector<double> last_dt;
  double *d_scratch = nullptr;
  // graphs of one full step: [0] from the caller's u, [1] from the scratch buffer
  cudaGraphExec_t step_graph[2] = {nullptr, nullptr};
  cudaStream_t capture_stream = nullptr;  // graphs are recorded here (the caller's stream may be the legacy one)
  const double *graph_u = nullptr;
  const double *graph_k = nullptr;
  // The groups of a step are independent chains of 5 stage launches, so the
  // step graph runs them as parallel branches (fork/join through events on
  // internal streams).  The branch count is picked by timing candidate graphs
  // once, on copies of the state, at the first graph build.
  int branches = 0;                        // 0: not tuned yet
  std::vector<int> tune_candidates;        // branch counts timed by the tuner
  std::vector<double> tune_ms;             // their ms per step
  std::vector<cudaStream_t> branch_streams;
  std::vector<cudaEvent_t> branch_events;  // [0] fork, [1 + j] join of branch j
  std::string last_error;
};

namespace {

int batch_fail(trixi_batch *b, int status, const std::string &msg) {
  g_last_error = msg;
  g_last_status = status;
  if (b) b->last_error = msg;
  return status;
}

struct KindKey {
  int32_t ndims, polydeg, eq, vol, vflux, sflux, fvflux, precision;
  double gamma, a0, a1, a2, amax, amin;
  int32_t smooth, ind_var;
  bool operator==(const KindKey &o) const {
    return ndims == o.ndims && polydeg == o.polydeg && eq == o.eq && vol == o.vol && vflux == o.vflux &&
           sflux == o.sflux && fvflux == o.fvflux && precision == o.precision && gamma == o.gamma && a0 == o.a0 &&
           a1 == o.a1 && a2 == o.a2 && amax == o.amax && amin == o.amin && smooth == o.smooth &&
           ind_var == o.ind_var;
  }
};

KindKey key_of(const trixi_problem_desc *d) {
  return KindKey{d->ndims, d->polydeg, d->equation, d->volume_integral, d->volume_flux, d->surface_flux,
                 d->volume_flux_fv, d->precision, d->gamma, d->advection_velocity[0], d->advection_velocity[1],
                 d->advection_velocity[2], d->alpha_max, d->alpha_min, d->alpha_smooth,
                 d->volume_integral == TRIXI_VOLUME_SHOCK_CAPTURING_HG ? d->indicator_variable : 0};
}

void destroy_graphs(trixi_batch *b) {
  for (auto &g : b->step_graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  b->graph_u = b->graph_k = nullptr;
}

// one full CK2N54 step of every group from `from` to `to` (5 stages ping-pong)
int batch_step(trixi_batch *b, double *from, double *to, double *k, cudaStream_t s) {
  double *cur = from, *nxt = to;
  for (int st = 0; st < 5; ++st) {
    for (auto &g : b->groups) {
      FusedHost save = g.h->fused;
      g.h->fused.dt_elem = g.d_dt;
      int r = run_rhs(g.h, MODE_RK, cur + g.value_offset, nxt + g.value_offset, k + g.value_offset, kCK_A[st],
                      kCK_B[st], 0.0, s);
      g.h->fused = save;
      if (r) return batch_fail(b, r, g.h->last_error);
    }
    std::swap(cur, nxt);
  }
  return TRIXI_OK;
}

// groups of each branch: longest-processing-time assignment by state size
std::vector<std::vector<int>> branch_groups(const trixi_batch *b, int nbranch) {
  std::vector<int> order(b->groups.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::sort(order.begin(), order.end(), [&](int x, int y) { return b->groups[x].nvalues > b->groups[y].nvalues; });
  std::vector<std::vector<int>> out((size_t)nbranch);
  std::vector<int64_t> load((size_t)nbranch, 0);
  for (int gi : order) {
    const size_t j = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
    out[j].push_back(gi);
    load[j] += b->groups[(size_t)gi].nvalues;
  }
  return out;
}

int ensure_branch_resources(trixi_batch *b, int nbranch) {
  while ((int)b->branch_streams.size() < nbranch) {
    cudaStream_t st = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    b->branch_streams.push_back(st);
  }
  while ((int)b->branch_events.size() < nbranch + 1) {
    cudaEvent_t ev = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    b->branch_events.push_back(ev);
  }
  return TRIXI_OK;
}

// One full step as `nbranch` parallel chains forked from and joined back into
// stream s (inside a capture on s this records a graph with parallel branches).
int batch_step_branched(trixi_batch *b, double *from, double *to, double *k, cudaStream_t s, int nbranch) {
  if (nbranch <= 1) return batch_step(b, from, to, k, s);
  if (int r = ensure_branch_resources(b, nbranch)) return r;
  const auto assign = branch_groups(b, nbranch);
  cudaError_t e = cudaEventRecord(b->branch_events[0], s);
  if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  for (int j = 0; j < nbranch; ++j) {
    cudaStream_t bs = b->branch_streams[(size_t)j];
    e = cudaStreamWaitEvent(bs, b->branch_events[0], 0);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    for (int gi : assign[(size_t)j]) {
      auto &g = b->groups[(size_t)gi];
      double *cur = from, *nxt = to;
      for (int st = 0; st < 5; ++st) {
        FusedHost save = g.h->fused;
        g.h->fused.dt_elem = g.d_dt;
        int r = run_rhs(g.h, MODE_RK, cur + g.value_offset, nxt + g.value_offset, k + g.value_offset, kCK_A[st],
                        kCK_B[st], 0.0, bs);
        g.h->fused = save;
        if (r) return batch_fail(b, r, g.h->last_error);
        std::swap(cur, nxt);
      }
    }
    e = cudaEventRecord(b->branch_events[(size_t)j + 1], bs);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    e = cudaStreamWaitEvent(s, b->branch_events[(size_t)j + 1], 0);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  }
  return TRIXI_OK;
}

// Captures one step from `from` to `to` with `nbranch` branches and instantiates it.
int capture_step(trixi_batch *b, double *from, double *to, double *k, int nbranch, cudaGraphExec_t *out) {
  cudaGraph_t graph = nullptr;
  cudaStream_t cs = b->capture_stream;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  int r = batch_step_branched(b, from, to, k, cs, nbranch);
  e = cudaStreamEndCapture(cs, &graph);
  if (r) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  e = cudaGraphInstantiate(out, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  return TRIXI_OK;
}

// Branch-count tuner: times one step graph per candidate on copies of u and k
// (the caller's data is not modified) and keeps the fastest.
int tune_branches(trixi_batch *b, const double *u, const double *k, cudaStream_t s) {
  const int G = (int)b->groups.size();
  std::vector<int> cand;
  for (int c : {1, 2, 4, 8, 16})
    if (c <= G) cand.push_back(c);
  if (G > 1 && std::find(cand.begin(), cand.end(), G) == cand.end() && G <= 32) cand.push_back(G);
  b->tune_candidates = cand;
  b->tune_ms.assign(cand.size(), 0.0);
  const size_t bytes = sizeof(double) * (size_t)b->total_values;
  double *tu = nullptr, *tk = nullptr;
  if (cudaMalloc(&tu, bytes) != cudaSuccess || cudaMalloc(&tk, bytes) != cudaSuccess) {
    if (tu) cudaFree(tu);
    cudaGetLastError();
    b->branches = std::min(G, 4);  // no room for the copies: a fixed choice
    return TRIXI_OK;
  }
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  int best = 1;
  double best_ms = 0.0;
  int status = TRIXI_OK;
  // first the tile of every group's kernel, on the copy of its state
  cudaMemcpyAsync(tu, u, bytes, cudaMemcpyDeviceToDevice, s);
  for (auto &g : b->groups) {
    if (status != TRIXI_OK) break;
    FusedHost save = g.h->fused;
    g.h->fused.dt_elem = g.d_dt;
    status = tune_tiles(g.h, tu + g.value_offset, s);
    const int w = g.h->fused.wpg, gg = g.h->fused.gpb;
    g.h->fused = save;
    g.h->fused.wpg = w;
    g.h->fused.gpb = gg;
    if (status != TRIXI_OK) status = batch_fail(b, status, g.h->last_error);
  }
  for (size_t ci = 0; ci < cand.size() && status == TRIXI_OK; ++ci) {
    cudaMemcpyAsync(tu, u, bytes, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(tk, k, bytes, cudaMemcpyDeviceToDevice, s);
    cudaGraphExec_t ge[2] = {nullptr, nullptr};
    status = capture_step(b, tu, b->d_scratch, tk, cand[ci], &ge[0]);
    if (status == TRIXI_OK) status = capture_step(b, b->d_scratch, tu, tk, cand[ci], &ge[1]);
    if (status == TRIXI_OK) {
      const int reps = 4;
      cudaGraphLaunch(ge[0], s);
      cudaGraphLaunch(ge[1], s);
      cudaEventRecord(t0, s);
      for (int r = 0; r < reps; ++r) {
        cudaGraphLaunch(ge[0], s);
        cudaGraphLaunch(ge[1], s);
      }
      cudaEventRecord(t1, s);
      cudaError_t e = cudaEventSynchronize(t1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
      if (e != cudaSuccess) status = batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
      b->tune_ms[ci] = ms / (2.0 * reps);
      if (ci == 0 || b->tune_ms[ci] < best_ms) {
        best = cand[ci];
        best_ms = b->tune_ms[ci];
      }
    }
    for (auto g : ge)
      if (g) cudaGraphExecDestroy(g);
  }
  cudaStreamSynchronize(s);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(tu);
  cudaFree(tk);
  if (status != TRIXI_OK) return status;
  b->branches = best;
  return TRIXI_OK;
}

}  // namespace

extern "C" {

int trixi_batch_create(const trixi_problem_desc *const *descs, int64_t n, trixi_batch **out) {
  if (!out || !descs || n <= 0) return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch: bad arguments");
  *out = nullptr;
  trixi_batch *b = new trixi_batch();
  std::vector<KindKey> keys;
  std::vector<std::vector<int64_t>> members;
  for (int64_t i = 0; i < n; ++i) {
    const trixi_problem_desc *d = descs[i];
    if (!d || d->struct_size != (int32_t)sizeof(trixi_problem_desc)) {
      delete b;
      return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch: instance " + std::to_string(i) + " descriptor");
    }
    if (d->equation == TRIXI_EQ_IDEAL_GLM_MHD) {
      delete b;
      return batch_fail(nullptr, TRIXI_ERR_UNSUPPORTED, "batch: ideal GLM-MHD instances are not batched");
    }
    const KindKey k = key_of(d);
    size_t gi = 0;
    while (gi < keys.size() && !(keys[gi] == k)) ++gi;
    if (gi == keys.size()) {
      keys.push_back(k);
      members.emplace_back();
    }
    members[gi].push_back(i);
  }
  if (keys.size() > 1)
    for (size_t gi = 1; gi < keys.size(); ++gi)
      if (keys[gi].precision != keys[0].precision) {
        delete b;
        return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch: mixed precisions in one batch");
      }
  b->inst_group.assign(n, 0);
  b->inst_offset.assign(n, 0);
  b->inst_nvalues.assign(n, 0);
  b->inst_nelem.assign(n, 0);
  int64_t offset = 0;
  for (size_t gi = 0; gi < keys.size(); ++gi) {
    const trixi_problem_desc *d0 = descs[members[gi][0]];
    const int nc = 1 << (d0->ndims - 1);
    int64_t nn = 1;
    for (int dd = 0; dd < d0->ndims; ++dd) nn *= d0->polydeg + 1;
    std::vector<double> inv_jac, coords;
    std::vector<int64_t> if_nid, if_ori, mo_nid, mo_ls, mo_ori;
    int64_t E = 0;
    bool have_coords = true;
    for (int64_t i : members[gi]) {
      const trixi_problem_desc *d = descs[i];
      if (d->nboundaries != 0 || !d->inverse_jacobian) {
        for (auto &g : b->groups) trixi_destroy(g.h);
        delete b;
        return batch_fail(nullptr, TRIXI_ERR_UNSUPPORTED, "batch: instance " + std::to_string(i));
      }
      b->inst_group[i] = (int64_t)gi;
      b->inst_nelem[i] = d->nelements;
      b->inst_nvalues[i] = d->nelements * nn * d->nvars;
      b->inst_offset[i] = offset + E * nn * d->nvars;
      inv_jac.insert(inv_jac.end(), d->inverse_jacobian, d->inverse_jacobian + d->nelements);
      if (d->node_coordinates)
        coords.insert(coords.end(), d->node_coordinates, d->node_coordinates + d->ndims * nn * d->nelements);
      else
        have_coords = false;
      for (int64_t k = 0; k < 2 * d->ninterfaces; ++k) if_nid.push_back(d->interface_neighbor_ids[k] + E);
      if_ori.insert(if_ori.end(), d->interface_orientations, d->interface_orientations + d->ninterfaces);
      for (int64_t k = 0; k < (nc + 1) * d->nmortars; ++k) mo_nid.push_back(d->mortar_neighbor_ids[k] + E);
      if (d->nmortars) {
        mo_ls.insert(mo_ls.end(), d->mortar_large_sides, d->mortar_large_sides + d->nmortars);
        mo_ori.insert(mo_ori.end(), d->mortar_orientations, d->mortar_orientations + d->nmortars);
      }
      E += d->nelements;
    }
    trixi_problem_desc md = *d0;
    md.nelements = E;
    md.inverse_jacobian = inv_jac.data();
    md.ninterfaces = (int64_t)if_ori.size();
    md.interface_neighbor_ids = if_nid.data();
    md.interface_orientations = if_ori.data();
    md.nmortars = (int64_t)mo_ori.size();
    md.mortar_neighbor_ids = mo_nid.empty() ? nullptr : mo_nid.data();
    md.mortar_large_sides = mo_ls.empty() ? nullptr : mo_ls.data();
    md.mortar_orientations = mo_ori.empty() ? nullptr : mo_ori.data();
    md.node_coordinates = have_coords ? coords.data() : nullptr;
    md.nghost_elements = 0;
    md.weights = md.derivative_split = md.derivative_dhat = md.inverse_vandermonde_legendre = nullptr;
    md.forward_upper = md.forward_lower = md.reverse_upper = md.reverse_lower = nullptr;
    trixi_batch::Group g;
    int st = trixi_create(&md, &g.h);
    if (st) {
      std::string msg = "batch group " + std::to_string(gi) + ": " + g_last_error;
      for (auto &gg : b->groups) trixi_destroy(gg.h);
      delete b;
      return batch_fail(nullptr, st, msg);
    }
    g.value_offset = offset;
    g.nvalues = E * nn * d0->nvars;
    g.instances = members[gi];
    if (cudaMalloc(&g.d_dt, sizeof(double) * (size_t)E) != cudaSuccess) {
      trixi_destroy(g.h);
      for (auto &gg : b->groups) trixi_destroy(gg.h);
      delete b;
      return batch_fail(nullptr, TRIXI_ERR_OUT_OF_MEMORY, "batch: dt buffer");
    }
    offset += g.nvalues;
    b->groups.push_back(g);
  }
  b->total_values = offset;
  *out = b;
  return TRIXI_OK;
}

int trixi_batch_destroy(trixi_batch *b) {
  if (!b) return TRIXI_OK;
  destroy_graphs(b);
  for (auto &g : b->groups) {
    if (g.d_dt) cudaFree(g.d_dt);
    trixi_destroy(g.h);
  }
  if (b->d_scratch) cudaFree(b->d_scratch);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  for (auto st : b->branch_streams) cudaStreamDestroy(st);
  for (auto ev : b->branch_events) cudaEventDestroy(ev);
  delete b;
  return TRIXI_OK;
}

int trixi_batch_tuning(const trixi_batch *b, int *branches, int *candidates, double *ms_per_step, int64_t max,
                       int64_t *count) {
  if (!b) return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch is null");
  if (branches) *branches = b->branches;
  const int64_t n = (int64_t)b->tune_candidates.size();
  if (count) *count = n;
  for (int64_t i = 0; i < n && i < max; ++i) {
    if (candidates) candidates[i] = b->tune_candidates[(size_t)i];
    if (ms_per_step) ms_per_step[i] = b->tune_ms[(size_t)i];
  }
  return TRIXI_OK;
}

int trixi_batch_layout(const trixi_batch *b, int64_t *value_offsets, int64_t *nvalues, int64_t *total_values,
                       int64_t *ngroups) {
  if (!b) return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch is null");
  const size_t n = b->inst_offset.size();
  for (size_t i = 0; i < n; ++i) {
    if (value_offsets) value_offsets[i] = b->inst_offset[i];
    if (nvalues) nvalues[i] = b->inst_nvalues[i];
  }
  if (total_values) *total_values = b->total_values;
  if (ngroups) *ngroups = (int64_t)b->groups.size();
  return TRIXI_OK;
}

int trixi_batch_rhs(trixi_batch *b, double *du, const double *u, void *stream) {
  if (!b) return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch is null");
  if (!aligned8(du) || !aligned8(u) || du == u) return batch_fail(b, TRIXI_ERR_INVALID_ARGUMENT, "batch rhs pointers");
  for (auto &g : b->groups) {
    int r = run_rhs(g.h, MODE_RHS, u + g.value_offset, du + g.value_offset, nullptr, 0, 0, 0, (cudaStream_t)stream);
    if (r) return batch_fail(b, r, g.h->last_error);
  }
  return TRIXI_OK;
}

int trixi_batch_rk_steps(trixi_batch *b, double *u, double *k, const double *dt_per_instance, int64_t nsteps,
                         int use_graph, void *stream) {
  if (!b) return batch_fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "batch is null");
  if (!aligned8(u) || !aligned8(k) || !dt_per_instance || nsteps < 0)
    return batch_fail(b, TRIXI_ERR_INVALID_ARGUMENT, "batch rk arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t ninst = b->inst_offset.size();
  if (b->last_dt.size() != ninst || !std::equal(b->last_dt.begin(), b->last_dt.end(), dt_per_instance)) {
    for (size_t i = 0; i < ninst; ++i)
      if (!std::isfinite(dt_per_instance[i])) return batch_fail(b, TRIXI_ERR_INVALID_ARGUMENT, "batch dt");
    for (auto &g : b->groups) {
      std::vector<double> dt;
      for (int64_t i : g.instances) dt.insert(dt.end(), (size_t)b->inst_nelem[i], dt_per_instance[i]);
      cudaError_t e = cudaMemcpy(g.d_dt, dt.data(), sizeof(double) * dt.size(), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    }
    b->last_dt.assign(dt_per_instance, dt_per_instance + ninst);
  }
  if (nsteps == 0) return TRIXI_OK;
  if (!b->d_scratch) {
    cudaError_t e = cudaMalloc(&b->d_scratch, sizeof(double) * (size_t)b->total_values);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_OUT_OF_MEMORY, "batch scratch");
  }
  double *bufs[2] = {u, b->d_scratch};
  if (use_graph && (b->graph_u != u || b->graph_k != k || !b->step_graph[0])) {
    destroy_graphs(b);
    if (!b->capture_stream) {
      cudaError_t e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    }
    // lazy initialisation (per-kernel shared-memory attributes) must not
    // happen during capture: a zero-element launch of every group's kernel
    // performs it without touching any data
    for (auto &g : b->groups) {
      FusedHost f = g.h->fused;
      f.nelements = 0;
      cudaError_t e = launch_fused(g.h->dim, g.h->N, g.h->eq, g.h->vol, g.h->vflux, g.h->mixed, f, s);
      if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    }
    if (b->branches == 0)
      if (int r = tune_branches(b, u, k, s)) return r;
    for (int parity = 0; parity < 2; ++parity)
      if (int r = capture_step(b, bufs[parity], bufs[1 - parity], k, b->branches, &b->step_graph[parity])) return r;
    b->graph_u = u;
    b->graph_k = k;
  }
  int cur = 0;
  for (int64_t st = 0; st < nsteps; ++st) {
    if (use_graph) {
      cudaError_t e = cudaGraphLaunch(b->step_graph[cur], s);
      if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
    } else {
      int r = batch_step(b, bufs[cur], bufs[1 - cur], k, s);
      if (r) return r;
    }
    cur = 1 - cur;
  }
  if (cur == 1) {
    cudaError_t e = cudaMemcpyAsync(u, b->d_scratch, sizeof(double) * (size_t)b->total_values,
                                    cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return batch_fail(b, TRIXI_ERR_CUDA, cudaGetErrorString(e));
  }
  return TRIXI_OK;
}

int trixi_batch_handle(trixi_batch *b, int64_t group, trixi_handle **h) {
  if (!b || !h || group < 0 || group >= (int64_t)b->groups.size())
    return batch_fail(b, TRIXI_ERR_INVALID_ARGUMENT, "batch group");
  *h = b->groups[(size_t)group].h;
  return TRIXI_OK;
}

int trixi_batch_last_error(const trixi_batch *b, char *buf, size_t len) {
  const std::string &msg = b ? b->last_error : g_last_error;
  if (buf && len > 0) {
    size_t m = std::min(len - 1, msg.size());
    std::memcpy(buf, msg.data(), m);
    buf[m] = '\0';
  }
  return TRIXI_OK;
}

}  // extern "C"

// ===========================================================================
// Discrete adjoint: VJP of the rhs, and reverse-mode CarpenterKennedy2N54 with
// binomial checkpointing (Griewank & Walther's "revolve" schedule: with s
// snapshots and r forward repetitions, beta(s, r) = C(s + r, s) steps can be
// reversed).  The forward sweep stores the snapshots of the schedule's
// rightmost branch; the backward sweep recomputes the rest.
// ===========================================================================
namespace {

AdjointHost adjoint_host(const trixi_handle *h) {
  AdjointHost a;
  a.dim = h->dim;
  a.N = h->N;
  a.eq = h->eq;
  a.vol = h->vol;
  a.face_table = h->d_face_table;
  a.inv_jac = h->d_inv_jac;
  a.nelements = h->E;
  a.surface_flux = h->sflux;
  a.volume_flux = h->vflux;
  a.gamma = h->gamma;
  for (int i = 0; i < 3; ++i) a.adv[i] = h->adv[i];
  for (int i = 0; i < h->N * h->N; ++i) {
    a.dsplit[i] = h->fused.dsplit[i];
    a.dhat[i] = h->fused.dhat[i];
  }
  a.lhat_l = h->fused.lhat_l;
  a.lhat_r = h->fused.lhat_r;
  a.pdl = h->fused.pdl;
  return a;
}

int check_adjoint_supported(trixi_handle *h) {
  if (h->eq == EQ_MHD) return fail(h, TRIXI_ERR_UNSUPPORTED, "adjoint: ideal GLM-MHD is not differentiated");
  if (h->mixed) return fail(h, TRIXI_ERR_UNSUPPORTED, "the adjoint runs in FP64 (precision = FP64)");
  if (h->B > 0 || h->src_kind != 0)
    return fail(h, TRIXI_ERR_UNSUPPORTED, "adjoint: periodic meshes without source terms only");
  if (!adjoint_supported(h->dim, h->N, h->eq, h->vol, h->vflux, h->sflux, h->M > 0))
    return fail(h, TRIXI_ERR_UNSUPPORTED,
                "adjoint: supported are Euler flux differencing with flux_ranocha/flux_central and linear "
                "advection, on conforming periodic meshes");
  return TRIXI_OK;
}

double beta(int64_t s, int64_t t) {  // C(s + t, s), saturating
  double r = 1.0;
  for (int64_t i = 1; i <= t; ++i) {
    r = r * (double)(s + i) / (double)i;
    if (r > 1e18) return 1e18;
  }
  return r;
}

// checkpoint position for reversing steps [a, b) with s free snapshots
int64_t split_point(int64_t a, int64_t b, int64_t s) {
  const int64_t n = b - a;
  if (s <= 0 || n <= 1) return -1;
  int64_t t = 1;
  while (beta(s, t) < (double)n) ++t;
  const double right = beta(s - 1, t);
  int64_t m = b - (int64_t)std::min<double>(right, (double)(n - 1));
  return std::max<int64_t>(a + 1, std::min<int64_t>(m, b - 1));
}

size_t state_bytes(const trixi_handle *h) { return sizeof(double) * (size_t)(h->E * h->NN * h->nv); }

// dst = state after `steps` RK steps from src (dst may equal src)
int advance(trixi_handle *h, const double *src, double *dst, int64_t steps, cudaStream_t s) {
  AdjointState *A = h->adj;
  if (src != dst) TRIXI_CUDA(h, cudaMemcpyAsync(dst, src, state_bytes(h), cudaMemcpyDeviceToDevice, s), "copy");
  if (steps > 0) {
    int r = trixi_rk_steps(h, dst, A->ktmp, 0.0, A->dt, steps, s);
    if (r) return r;
    A->fwd_steps += steps;
  }
  return TRIXI_OK;
}

int adjoint_step(trixi_handle *h, const double *state, int &cur, cudaStream_t s) {
  AdjointState *A = h->adj;
  TRIXI_CUDA(h, cudaMemcpyAsync(A->stage[0], state, state_bytes(h), cudaMemcpyDeviceToDevice, s), "copy");
  for (int st = 0; st < 4; ++st) {
    int r = run_rhs(h, MODE_RK, A->stage[st], A->stage[st + 1], A->ktmp, kCK_A[st], kCK_B[st], A->dt, s);
    if (r) return r;
  }
  AdjointHost a = adjoint_host(h);
  a.dt = A->dt;
  for (int st = 4; st >= 0; --st) {
    a.u = A->stage[st];
    a.lu_in = A->lu[cur];
    a.lk_in = A->lk[cur];
    a.lu_out = A->lu[1 - cur];
    a.lk_out = A->lk[1 - cur];
    a.rk_a = kCK_A[st];
    a.rk_b = kCK_B[st];
    TRIXI_CUDA(h, launch_adjoint(a, s), "adjoint stage");
    cur = 1 - cur;
  }
  return TRIXI_OK;
}

int reverse(trixi_handle *h, int64_t a, int64_t b, int64_t s_free, const double *state_a, int &cur, cudaStream_t st) {
  AdjointState *A = h->adj;
  if (b - a == 1) return adjoint_step(h, state_a, cur, st);
  const int64_t m = split_point(a, b, s_free);
  if (m < 0) {  // no snapshot left: recompute every step from a
    for (int64_t j = b - 1; j >= a; --j) {
      int r = advance(h, state_a, A->tmp, j - a, st);
      if (r) return r;
      r = adjoint_step(h, A->tmp, cur, st);
      if (r) return r;
    }
    return TRIXI_OK;
  }
  double *buf = nullptr;
  auto it = A->ckpt.find(m);
  if (it != A->ckpt.end()) {
    buf = it->second;
  } else {
    if (A->pool.empty()) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "adjoint: snapshot pool exhausted");
    buf = A->pool.back();
    A->pool.pop_back();
    int r = advance(h, state_a, buf, m - a, st);
    if (r) return r;
    A->ckpt[m] = buf;
  }
  int r = reverse(h, m, b, s_free - 1, buf, cur, st);
  if (r) return r;
  A->ckpt.erase(m);
  A->pool.push_back(buf);
  return reverse(h, a, m, s_free, state_a, cur, st);
}

}  // namespace

extern "C" {

int trixi_rhs_vjp(trixi_handle *h, double *ubar, const double *u, const double *lambda, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, ubar, "ubar")) return st;
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_u_args(h, lambda, "lambda")) return st;
  if (int st = check_adjoint_supported(h)) return st;
  AdjointHost a = adjoint_host(h);
  a.u = u;
  a.lu_in = nullptr;
  a.lk_in = lambda;
  a.lu_out = ubar;
  a.lk_out = nullptr;
  a.rk_a = 0.0;
  a.rk_b = 0.0;
  a.dt = 1.0;
  TRIXI_CUDA(h, launch_adjoint(a, (cudaStream_t)stream), "rhs vjp");
  return TRIXI_OK;
}

int trixi_objective_density_l2(trixi_handle *h, const double *u, const double *rho_target, double *J_host,
                               double *ubar, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u, "u")) return st;
  if (int st = check_u_args(h, rho_target, "rho_target")) return st;
  if (!J_host) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "J is null");
  if (ubar && !aligned8(ubar)) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "ubar misaligned");
  if (int st = ensure_reduction(h, 1)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  TRIXI_CUDA(h, launch_density_objective(h->dim, h->N, h->nv, h->E, u, rho_target, h->d_inv_jac, h->d_w, ubar,
                                         h->d_partial, h->d_red_out, s), "objective");
  TRIXI_CUDA(h, cudaMemcpyAsync(J_host, h->d_red_out, sizeof(double), cudaMemcpyDeviceToHost, s), "copy");
  TRIXI_CUDA(h, cudaStreamSynchronize(s), "synchronize");
  return TRIXI_OK;
}

int trixi_adjoint_forward(trixi_handle *h, const double *u0, double dt, int64_t nsteps, int64_t nsnapshots,
                          double *uT, void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (int st = check_u_args(h, u0, "u0")) return st;
  if (int st = check_u_args(h, uT, "uT")) return st;
  if (int st = check_adjoint_supported(h)) return st;
  if (nsteps <= 0 || nsnapshots < 0 || !std::isfinite(dt))
    return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "adjoint: nsteps %lld, snapshots %lld", (long long)nsteps,
                (long long)nsnapshots);
  cudaStream_t s = (cudaStream_t)stream;
  free_adjoint(h);
  h->adj = new AdjointState();
  AdjointState *A = h->adj;
  A->n = nsteps;
  A->snapshots = std::min<int64_t>(nsnapshots, nsteps - 1);
  A->dt = dt;
  const size_t bytes = state_bytes(h);
  auto alloc = [&](double **p) -> int {
    TRIXI_CUDA(h, cudaMalloc(p, bytes), "alloc adjoint buffers");
    A->all.push_back(*p);
    return TRIXI_OK;
  };
  int r = alloc(&A->u0);
  if (!r) r = alloc(&A->ktmp);
  if (!r) r = alloc(&A->tmp);
  for (int i = 0; i < 5 && !r; ++i) r = alloc(&A->stage[i]);
  for (int i = 0; i < 2 && !r; ++i) r = alloc(&A->lu[i]);
  for (int i = 0; i < 2 && !r; ++i) r = alloc(&A->lk[i]);
  // store-all mode: when the snapshot budget covers every step and the stage
  // states of the whole solve fit in half of the free memory, keep the input
  // of every RK stage, so that the backward sweep recomputes nothing
  if (!r && nsnapshots >= nsteps - 1) {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t need = 5 * (size_t)nsteps * bytes;
    if (need < free_b / 2 && cudaMalloc(&A->stages_all, need) == cudaSuccess) A->all.push_back(A->stages_all);
  }
  for (int64_t i = 0; i < A->snapshots && !r && !A->stages_all; ++i) {
    double *p = nullptr;
    r = alloc(&p);
    if (!r) A->pool.push_back(p);
  }
  if (r) {
    free_adjoint(h);
    return r;
  }
  TRIXI_CUDA(h, cudaMemcpyAsync(A->u0, u0, bytes, cudaMemcpyDeviceToDevice, s), "copy u0");
  if (A->stages_all) {
    {
      const size_t nval = bytes / sizeof(double);
      TRIXI_CUDA(h, cudaMemcpyAsync(A->stages_all, A->u0, bytes, cudaMemcpyDeviceToDevice, s), "copy");
      for (int64_t j = 0; j < nsteps; ++j) {
        double *base = A->stages_all + (size_t)j * 5 * nval;
        for (int st = 0; st < 5; ++st) {
          double *out = (st < 4) ? base + (size_t)(st + 1) * nval : (j + 1 < nsteps ? base + 5 * nval : uT);
          r = run_rhs(h, MODE_RK, base + (size_t)st * nval, out, A->ktmp, kCK_A[st], kCK_B[st], dt, s);
          if (r) return r;
        }
      }
      A->fwd_steps = 0;
      A->forward_done = true;
      return TRIXI_OK;
    }
  }
  // forward sweep to T, storing the snapshots of the schedule's rightmost branch
  int64_t a = 0, s_free = A->snapshots;
  const double *from = A->u0;
  TRIXI_CUDA(h, cudaMemcpyAsync(uT, A->u0, bytes, cudaMemcpyDeviceToDevice, s), "copy");
  int64_t pos = 0;
  while (true) {
    const int64_t m = split_point(a, nsteps, s_free);
    if (m < 0) break;
    double *buf = A->pool.back();
    A->pool.pop_back();
    r = advance(h, from, buf, m - pos, s);
    if (r) return r;
    A->ckpt[m] = buf;
    from = buf;
    pos = m;
    a = m;
    --s_free;
  }
  r = advance(h, from, uT, nsteps - pos, s);
  if (r) return r;
  A->fwd_steps = 0;  // count only the recomputation of the backward sweep
  A->forward_done = true;
  return TRIXI_OK;
}

int trixi_adjoint_backward(trixi_handle *h, const double *uT_bar, double *u0_bar, int64_t *forward_steps,
                           void *stream) {
  if (!h) return fail(nullptr, TRIXI_ERR_INVALID_ARGUMENT, "handle is null");
  if (!h->adj || !h->adj->forward_done) return fail(h, TRIXI_ERR_INVALID_ARGUMENT, "adjoint: run the forward sweep first");
  if (int st = check_u_args(h, uT_bar, "uT_bar")) return st;
  if (int st = check_u_args(h, u0_bar, "u0_bar")) return st;
  cudaStream_t s = (cudaStream_t)stream;
  AdjointState *A = h->adj;
  const size_t bytes = state_bytes(h);
  int cur = 0;
  TRIXI_CUDA(h, cudaMemcpyAsync(A->lu[0], uT_bar, bytes, cudaMemcpyDeviceToDevice, s), "copy");
  TRIXI_CUDA(h, cudaMemsetAsync(A->lk[0], 0, bytes, s), "zero");
  int r = TRIXI_OK;
  if (A->stages_all) {
    const size_t nval = bytes / sizeof(double);
    AdjointHost adj = adjoint_host(h);
    adj.dt = A->dt;
    adj.u_ready = 1;  // the stored stage states were written by the forward sweep, before these launches
    for (int64_t j = A->n - 1; j >= 0; --j)
      for (int st = 4; st >= 0; --st) {
        adj.u = A->stages_all + ((size_t)j * 5 + st) * nval;
        adj.lu_in = A->lu[cur];
        adj.lk_in = A->lk[cur];
        adj.lu_out = A->lu[1 - cur];
        adj.lk_out = A->lk[1 - cur];
        adj.rk_a = kCK_A[st];
        adj.rk_b = kCK_B[st];
        TRIXI_CUDA(h, launch_adjoint(adj, s), "adjoint stage");
        cur = 1 - cur;
      }
  } else {
    r = reverse(h, 0, A->n, A->snapshots, A->u0, cur, s);
  }
  if (r) return r;
  TRIXI_CUDA(h, cudaMemcpyAsync(u0_bar, A->lu[cur], bytes, cudaMemcpyDeviceToDevice, s), "copy");
  if (forward_steps) *forward_steps = A->fwd_steps;
  A->forward_done = false;
  return TRIXI_OK;
}

}  // extern "C"
