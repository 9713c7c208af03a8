"""SemidiscretizationHyperbolicGPU, semidiscretizeGPU, rhs_gpu and the stage
functions -- the host side of the reference's public API, backed by
libtrixi_b200.so.

Reference interfaces mirrored here:
  SemidiscretizationHyperbolicGPU  src/semidiscretization/semidiscretization_hyperbolic.jl:60-87
  semidiscretizeGPU                src/solvers/solvers.jl:43-56
  rhs_gpu!(du_ode, u_ode, semi, t) src/solvers/solvers.jl:18-31
  wrap_array                       src/solvers/dg.jl:14-20
  cuda_* stage functions           src/solvers/dg_{1,2,3}d.jl, docstrings dg.jl:164-325

Device arrays are torch CUDA tensors (float64) in the reference layout
[nvars, N, ..., nelements] column-major, i.e. C-order shape
(nelements, N, ..., nvars).  Compute calls go through the C ABI on the
current torch stream; none of them has a CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from .equations import AbstractEquations, flux_lax_friedrichs
from .mesh import Containers, TreeMesh
from .solver import DGSEMGPU, VolumeIntegralShockCapturingHG, VolumeIntegralFluxDifferencing


def _torch():
    import torch

    return torch


def _ptr_d(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a.size else None


def _ptr_i(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64)) if a.size else None


def _stream_handle(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _boundary_spec(boundary_conditions, cont, equations):
    """(code, params) of the Dirichlet boundary function, or (-1, None) on a
    periodic mesh.  One boundary function serves every non-periodic direction."""
    from .equations import BoundaryConditionDirichlet, boundary_function_code

    if cont.nboundaries == 0:
        return -1, None
    bcs = boundary_conditions
    if isinstance(bcs, dict):
        vals = list(bcs.values())
    elif isinstance(bcs, (tuple, list)):
        vals = list(bcs)
    else:
        vals = [bcs]
    vals = [b for b in vals if b not in ("periodic", None)]
    if not vals or not all(isinstance(b, BoundaryConditionDirichlet) for b in vals) or any(b != vals[0] for b in vals):
        raise NotImplementedError("non-periodic meshes need one BoundaryConditionDirichlet for all boundaries")
    code = boundary_function_code(vals[0].boundary_value_function)
    params = None
    if code == _lib.IC_CONSTANT:
        x = np.zeros((equations.ndims, 1))
        params = np.asarray(vals[0].boundary_value_function(x, 0.0, equations))[:, 0]
        if params.size > 8:
            raise NotImplementedError(f"a constant Dirichlet state of {params.size} variables: the problem "
                                      "descriptor holds 8 boundary parameters")
    return code, params


def flux_codes(solver: DGSEMGPU, equations: AbstractEquations) -> dict:
    """Enum codes of the solver's fluxes.  Equations with nonconservative
    terms (ideal GLM-MHD in 2D/3D) take every flux as a `(flux,
    nonconservative_flux)` pair with one common nonconservative flux, as
    Trixi's do; the others take plain fluxes."""
    from .equations import split_flux

    vi = solver.volume_integral
    pairs = {"surface_flux": solver.surface_flux}
    if isinstance(vi, VolumeIntegralFluxDifferencing):
        pairs["volume_flux"] = vi.volume_flux
    if isinstance(vi, VolumeIntegralShockCapturingHG):
        pairs["volume_flux"] = vi.volume_flux_dg
        pairs["volume_flux_fv"] = vi.volume_flux_fv
    out = {"volume_flux": _lib.FLUX_CENTRAL, "volume_flux_fv": _lib.FLUX_LAX_FRIEDRICHS}
    nc = set()
    for k, f in pairs.items():
        sym, ncf = split_flux(f)
        out[k] = sym.code
        nc.add(ncf.code if ncf is not None else _lib.NONCONSERVATIVE_NONE)
    need = bool(getattr(equations, "have_nonconservative_terms", False))
    if len(nc) != 1 or (need and _lib.NONCONSERVATIVE_NONE in nc) or (not need and nc != {_lib.NONCONSERVATIVE_NONE}):
        raise ValueError(f"{equations!r} takes {'(flux, nonconservative_flux) pairs' if need else 'plain fluxes'} "
                         "for every volume and surface flux")
    out["nonconservative_flux"] = nc.pop()
    return out


def build_problem_desc(mesh_or_containers, equations: AbstractEquations, solver: DGSEMGPU,
                       precision: str = "fp64", boundary_conditions="periodic", source_terms=None):
    """trixi_problem_desc for a mesh (or prebuilt containers).  Returns the
    ctypes struct and the numpy arrays it points into (keep them alive)."""
    if isinstance(mesh_or_containers, Containers):
        cont = mesh_or_containers
    else:
        cont = mesh_or_containers.build_containers(solver.basis.nodes)
    d = _lib.ProblemDesc()
    d.struct_size = C.sizeof(_lib.ProblemDesc)
    d.ndims = cont.ndims
    d.polydeg = solver.polydeg
    d.nvars = equations.nvariables
    d.equation = equations.code
    vi = solver.volume_integral
    d.volume_integral = vi.code
    codes = flux_codes(solver, equations)
    d.volume_flux, d.surface_flux, d.volume_flux_fv = codes["volume_flux"], codes["surface_flux"], codes["volume_flux_fv"]
    d.nonconservative_flux = codes["nonconservative_flux"]
    d.glm_speed = float(getattr(equations, "c_h", 0.0))
    d.alpha_max, d.alpha_min, d.alpha_smooth = 0.5, 0.001, 1
    if isinstance(vi, VolumeIntegralShockCapturingHG):
        d.alpha_max = vi.indicator.alpha_max
        d.alpha_min = vi.indicator.alpha_min
        d.alpha_smooth = int(bool(vi.indicator.alpha_smooth))
        d.indicator_variable = vi.indicator.variable_code
    if precision not in ("fp64", "mixed"):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    d.precision = _lib.PRECISION_MIXED if precision == "mixed" else _lib.PRECISION_FP64
    d.gamma = float(getattr(equations, "gamma", 1.4))
    av = np.zeros(3)
    av[: equations.ndims] = getattr(equations, "advection_velocity", np.zeros(equations.ndims))
    for i in range(3):
        d.advection_velocity[i] = av[i]
    keep = dict(
        inverse_jacobian=np.ascontiguousarray(cont.inverse_jacobian, dtype=np.float64),
        if_nid=np.ascontiguousarray(cont.interface_neighbor_ids, dtype=np.int64),
        if_ori=np.ascontiguousarray(cont.interface_orientations, dtype=np.int64),
        mo_nid=np.ascontiguousarray(cont.mortar_neighbor_ids, dtype=np.int64),
        mo_ls=np.ascontiguousarray(cont.mortar_large_sides, dtype=np.int64),
        mo_ori=np.ascontiguousarray(cont.mortar_orientations, dtype=np.int64),
        coords=np.ascontiguousarray(cont.node_coordinates, dtype=np.float64),
    )
    d.nelements = cont.nelements
    d.inverse_jacobian = _ptr_d(keep["inverse_jacobian"])
    d.ninterfaces = cont.ninterfaces
    d.interface_neighbor_ids = _ptr_i(keep["if_nid"])
    d.interface_orientations = _ptr_i(keep["if_ori"])
    d.nboundaries = 0
    d.nmortars = cont.nmortars
    d.mortar_neighbor_ids = _ptr_i(keep["mo_nid"])
    d.mortar_large_sides = _ptr_i(keep["mo_ls"])
    d.mortar_orientations = _ptr_i(keep["mo_ori"])
    d.node_coordinates = _ptr_d(keep["coords"])
    d.nghost_elements = int(getattr(cont, "nghost_elements", 0))
    # non-periodic meshes and source terms
    keep["b_nid"] = np.ascontiguousarray(cont.boundary_neighbor_ids, dtype=np.int64)
    keep["b_side"] = np.ascontiguousarray(cont.boundary_neighbor_sides, dtype=np.int64)
    keep["b_ori"] = np.ascontiguousarray(cont.boundary_orientations, dtype=np.int64)
    d.nboundaries = cont.nboundaries
    d.boundary_neighbor_ids = _ptr_i(keep["b_nid"])
    d.boundary_neighbor_sides = _ptr_i(keep["b_side"])
    d.boundary_orientations = _ptr_i(keep["b_ori"])
    code, params = _boundary_spec(boundary_conditions, cont, equations)
    d.boundary_function = code
    d.nboundary_params = 0 if params is None else len(params)
    for i in range(d.nboundary_params):
        d.boundary_params[i] = float(params[i])
    from .equations import source_terms_convergence_test, source_terms_eoc_test_euler

    if source_terms is None:
        d.source_terms = _lib.SOURCE_NONE
    elif source_terms is source_terms_convergence_test:
        d.source_terms = _lib.SOURCE_CONVERGENCE_TEST
    elif source_terms is source_terms_eoc_test_euler:
        d.source_terms = _lib.SOURCE_EOC_TEST_EULER
    else:
        raise NotImplementedError("source terms: source_terms_convergence_test or source_terms_eoc_test_euler; "
                                  "other Julia source callables cannot cross the C ABI")
    d.nsource_params = 0
    return d, keep, cont


class SemidiscretizationHyperbolicGPU:
    """GPU semidiscretization (reference:
    src/semidiscretization/semidiscretization_hyperbolic.jl:5-87)."""

    def __init__(self, mesh: TreeMesh, equations: AbstractEquations, initial_condition, solver: DGSEMGPU,
                 source_terms=None, boundary_conditions="periodic", RealT=np.float64, uEltype=np.float64,
                 precision: str = "fp64", device=None, containers=None):
        if mesh.ndims != equations.ndims:
            raise ValueError("mesh and equations dimension differ")
        self.mesh = mesh
        self.equations = equations
        self.initial_condition = initial_condition
        self.solver = solver
        self.source_terms = source_terms
        self.boundary_conditions = boundary_conditions
        self.precision = precision
        desc, keep, cont = build_problem_desc(containers if containers is not None else mesh, equations, solver,
                                              precision, boundary_conditions, source_terms)
        self.containers = cont
        self._desc, self._keep = desc, keep
        torch = _torch()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        lib = _lib.load()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.trixi_create(C.byref(desc), C.byref(h)))
        self._handle = h
        self._lib = lib

    # -- sizes -------------------------------------------------------------
    @property
    def handle(self):
        return self._handle

    @property
    def nnodes(self) -> int:
        return self.solver.polydeg + 1

    @property
    def nelements(self) -> int:
        return self.containers.nelements

    def ndofs(self) -> int:
        """Nodes per field, Trixi's ndofsglobal (benchmark/euler_ec_2d.jl:65)."""
        return self.nelements * self.nnodes ** self.mesh.ndims

    def u_shape(self):
        return (self.nelements,) + (self.nnodes,) * self.mesh.ndims + (self.equations.nvariables,)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.trixi_destroy(h)
            except Exception:
                pass
            self._handle = None

    # -- initial data ------------------------------------------------------
    def compute_coefficients_host(self, t: float = 0.0, func=None) -> np.ndarray:
        """u0 on the host in the reference layout, evaluating the initial
        condition at every node (reference: compute_coefficients_kernel!,
        src/solvers/dg.jl:46-115, including the 1D endpoint nudge of x by one
        ulp inward, dg.jl:54-57)."""
        func = func or self.initial_condition
        d = self.mesh.ndims
        x = self.containers.node_coordinates.reshape(-1, d).T.copy()
        if d == 1:
            N = self.nnodes
            x1 = x.reshape(1, -1, N)
            x1[0, :, 0] = np.nextafter(x1[0, :, 0], np.inf)
            x1[0, :, N - 1] = np.nextafter(x1[0, :, N - 1], -np.inf)
            x = x1.reshape(1, -1)
        u = func(x, t, self.equations)  # (nvars, nnodes_total)
        return np.ascontiguousarray(u.T.reshape(self.u_shape()))

    def compute_coefficients(self, t: float = 0.0, func=None):
        torch = _torch()
        return torch.from_numpy(self.compute_coefficients_host(t, func)).to(self.device)

    # -- containers ----------------------------------------------------------
    def container(self, which: int):
        """A library-owned device container as a torch tensor view (no copy)."""
        torch = _torch()
        ptr, cnt = C.c_void_p(), C.c_int64()
        _lib.check(self._lib.trixi_container(self._handle, which, C.byref(ptr), C.byref(cnt)), self._handle)
        if cnt.value == 0 or not ptr.value:
            return torch.empty(0, dtype=torch.float64, device=self.device)
        # wrap the device pointer through a DLPack-free route: cupy-less torch view
        return _device_view(ptr.value, cnt.value, self.device)


def set_glm_speed(semi, c_h: float) -> None:
    """Set the GLM cleaning speed c_h of an ideal GLM-MHD semidiscretization
    (what Trixi's GlmSpeedCallback does to `equations.c_h` between steps)."""
    c_h = float(c_h)
    _lib.check(semi._lib.trixi_set_glm_speed(semi._handle, c_h), semi._handle)
    semi.equations.c_h = c_h


def _device_view(ptr: int, count: int, device):
    """Torch tensor aliasing `count` float64 values at device pointer `ptr`."""
    torch = _torch()

    class _CudaArray:
        def __init__(self, p, n):
            self.__cuda_array_interface__ = {
                "shape": (n,), "typestr": "<f8", "data": (p, False), "version": 2, "strides": None,
            }

    return torch.as_tensor(_CudaArray(ptr, count), device=device)


def wrap_array(u_ode, semi: SemidiscretizationHyperbolicGPU):
    """Reshape a flat state vector to [nvars, N, ..., nelements] (C-order
    view (nelements, N, ..., nvars)); reference src/solvers/dg.jl:14-20."""
    return u_ode.view(semi.u_shape())


@dataclass
class ODEProblem:
    f: object
    u0: object
    tspan: tuple
    p: SemidiscretizationHyperbolicGPU


def _check_state(semi, *arrays):
    torch = _torch()
    n = int(math.prod(semi.u_shape()))  # (np.prod costs ~3 us per call, on every rhs)
    for a in arrays:
        if not isinstance(a, torch.Tensor) or a.dtype != torch.float64 or not a.is_cuda:
            raise TypeError("state arrays must be float64 CUDA tensors")
        if a.numel() != n or not a.is_contiguous():
            raise ValueError(f"state array must be contiguous with {n} values")


def rhs_gpu(du_ode, u_ode, semi: SemidiscretizationHyperbolicGPU, t: float, stream=None):
    """du = rhs(u, t) on the GPU, in place (reference rhs_gpu!, solvers.jl:18-31)."""
    _check_state(semi, du_ode, u_ode)
    _lib.check(semi._lib.trixi_rhs(semi._handle, C.c_void_p(du_ode.data_ptr()), C.c_void_p(u_ode.data_ptr()),
                                   float(t), _stream_handle(stream)), semi._handle)


def semidiscretizeGPU(semi: SemidiscretizationHyperbolicGPU, tspan):
    """ODE problem with u0 on the GPU (reference semidiscretizeGPU, solvers.jl:43-56)."""
    u0 = semi.compute_coefficients(float(tspan[0])).reshape(-1)
    return ODEProblem(rhs_gpu, u0, (float(tspan[0]), float(tspan[1])), semi)


# -- stage functions (reference cuda_* launchers) ---------------------------------
def _call(semi, fn, *args, stream=None):
    _lib.check(fn(semi._handle, *args, _stream_handle(stream)), semi._handle)


def cuda_volume_integral(du, u, semi, stream=None):
    _check_state(semi, du, u)
    _call(semi, semi._lib.trixi_volume_integral, C.c_void_p(du.data_ptr()), C.c_void_p(u.data_ptr()), stream=stream)


def cuda_prolong2interfaces(u, semi, stream=None):
    _check_state(semi, u)
    _call(semi, semi._lib.trixi_prolong2interfaces, C.c_void_p(u.data_ptr()), stream=stream)


def cuda_interface_flux(semi, stream=None):
    _call(semi, semi._lib.trixi_interface_flux, stream=stream)


def cuda_prolong2boundaries(u, semi, stream=None):
    _check_state(semi, u)
    _call(semi, semi._lib.trixi_prolong2boundaries, C.c_void_p(u.data_ptr()), stream=stream)


def cuda_boundary_flux(t, semi, stream=None):
    _call(semi, semi._lib.trixi_boundary_flux, float(t), stream=stream)


def cuda_prolong2mortars(u, semi, stream=None):
    _check_state(semi, u)
    _call(semi, semi._lib.trixi_prolong2mortars, C.c_void_p(u.data_ptr()), stream=stream)


def cuda_mortar_flux(semi, stream=None):
    _call(semi, semi._lib.trixi_mortar_flux, stream=stream)


def cuda_surface_integral(du, semi, stream=None):
    _check_state(semi, du)
    _call(semi, semi._lib.trixi_surface_integral, C.c_void_p(du.data_ptr()), stream=stream)


def cuda_jacobian(du, semi, stream=None):
    _check_state(semi, du)
    _call(semi, semi._lib.trixi_jacobian, C.c_void_p(du.data_ptr()), stream=stream)


def cuda_sources(du, u, t, semi, stream=None):
    _check_state(semi, du, u)
    _call(semi, semi._lib.trixi_sources, C.c_void_p(du.data_ptr()), C.c_void_p(u.data_ptr()), float(t),
          stream=stream)


def cuda_indicator(u, alpha, semi, stream=None):
    """Hennemann-Gassner blending factors on the GPU into `alpha` (float64, nelements)."""
    _check_state(semi, u)
    _call(semi, semi._lib.trixi_indicator, C.c_void_p(u.data_ptr()), C.c_void_p(alpha.data_ptr()), stream=stream)


def rk_stage(u_out, u_in, k, a, b, dt, t, semi, stream=None):
    _check_state(semi, u_out, u_in, k)
    _call(semi, semi._lib.trixi_rk_stage, C.c_void_p(u_out.data_ptr()), C.c_void_p(u_in.data_ptr()),
          C.c_void_p(k.data_ptr()), float(a), float(b), float(dt), float(t), stream=stream)


def rk_steps(u, k, t, dt, nsteps, semi, stream=None):
    _check_state(semi, u, k)
    _call(semi, semi._lib.trixi_rk_steps, C.c_void_p(u.data_ptr()), C.c_void_p(k.data_ptr()), float(t),
          float(dt), int(nsteps), stream=stream)


def rk_steps_host(u_in, u_out, t, dt, nsteps, semi, stream=None, wait_event=None, done_event=None):
    """rk_steps on a state in host memory (C ABI trixi_rk_steps_host): u_in
    is uploaded to a library-owned device buffer, advanced nsteps
    CarpenterKennedy2N54 steps and downloaded to u_out, all enqueued on
    `stream`.  u_in / u_out: contiguous float64 CPU tensors (page-locked for
    an asynchronous call: synchronise before reading u_out) or numpy arrays;
    wait_event / done_event: optional torch.cuda.Event ordering hooks (the
    stream waits for wait_event before the first stage; done_event is
    recorded after the last one)."""
    torch = _torch()
    n = int(math.prod(semi.u_shape()))

    def ptr(a, what):
        if isinstance(a, torch.Tensor):
            if a.is_cuda or a.dtype != torch.float64 or not a.is_contiguous() or a.numel() != n:
                raise ValueError(f"{what}: a contiguous float64 CPU tensor with {n} values is required")
            return C.c_void_p(a.data_ptr())
        if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous or a.size != n:
            raise ValueError(f"{what}: a contiguous float64 array with {n} values is required")
        return C.c_void_p(a.ctypes.data)

    def ev(e):
        return C.c_void_p(e.cuda_event) if e is not None else None

    _call(semi, semi._lib.trixi_rk_steps_host, ptr(u_in, "u_in"), ptr(u_out, "u_out"), float(t), float(dt),
          int(nsteps), ev(wait_event), ev(done_event), stream=stream)


def autotune(u, semi, stream=None):
    """Picks the fused kernel's tile (warps per element group, groups per
    block) for this problem by timing every valid tile on u (read only)."""
    _check_state(semi, u)
    _call(semi, semi._lib.trixi_autotune, C.c_void_p(u.data_ptr()), stream=stream)


def set_tile(semi, wpg, gpb):
    """Fixes the tile by hand; wpg = gpb = 0 restores the compile-time default."""
    _lib.check(semi._lib.trixi_set_tile(semi._handle, int(wpg), int(gpb)), semi._handle)


def _read_tile(lib, handle):
    epg, wpg, gpb, cnt = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
    cw, cg, cm = (C.c_int * 64)(), (C.c_int * 64)(), (C.c_double * 64)()
    _lib.check(lib.trixi_tile(handle, C.byref(epg), C.byref(wpg), C.byref(gpb), cw, cg, cm, 64, C.byref(cnt)),
               handle)
    n = min(int(cnt.value), 64)
    return (int(epg.value), int(wpg.value), int(gpb.value)), {(int(cw[i]), int(cg[i])): float(cm[i]) for i in range(n)}


def tile(semi):
    """((elements per group, warps per group, groups per block), the tuner's
    {(wpg, gpb): ms per launch}) -- the table is empty before autotune."""
    return _read_tile(semi._lib, semi._handle)


# -- analysis, time step and initial conditions on the GPU (reference callbacks) ----
_IC_KINDS = {"constant": _lib.IC_CONSTANT, "convergence_test": _lib.IC_CONVERGENCE_TEST,
             "weak_blast_wave": _lib.IC_WEAK_BLAST_WAVE,
             "eoc_test_coupled_euler_gravity": _lib.IC_EOC_TEST_COUPLED_EULER_GRAVITY}


def _ic_args(kind, params):
    code = _IC_KINDS[kind] if isinstance(kind, str) else int(kind)
    if params is None:
        return code, None, 0, None
    arr = np.ascontiguousarray(params, dtype=np.float64)
    return code, arr.ctypes.data_as(C.POINTER(C.c_double)), arr.size, arr


def compute_coefficients_gpu(semi, kind, t=0.0, params=None, out=None, stream=None):
    """u0 = initial condition evaluated on the GPU (reference compute_coefficients_gpu,
    src/semidiscretization/semidiscretization.jl:4-20, dg.jl:46-160)."""
    torch = _torch()
    u = out if out is not None else torch.empty(semi.u_shape(), dtype=torch.float64, device=semi.device)
    code, ptr, n, keep = _ic_args(kind, params)
    _call(semi, semi._lib.trixi_compute_coefficients, code, ptr, n, float(t), C.c_void_p(u.data_ptr()),
          stream=stream)
    return u


def max_dt(u, semi, stream=None) -> float:
    """2 / (N max_e J^{-1} sum_d max lambda_d) on the GPU (reference max_dt,
    src/callbacks_step/stepsize_dg_2d.jl:21-45); multiply by the CFL number."""
    torch = _torch()
    _check_state(semi, u)
    dt = torch.empty(1, dtype=torch.float64, device=semi.device)
    _call(semi, semi._lib.trixi_max_dt, C.c_void_p(u.data_ptr()), C.c_void_p(dt.data_ptr()), stream=stream)
    return float(dt.item())


def integrate(u, semi, which="state", du=None, stream=None) -> np.ndarray:
    """sum_e J_e sum_nodes w q (reference integrate_via_indices,
    src/callbacks_step/analysis_dg_2d.jl:1-40, without the volume normalisation)."""
    codes = {"state": _lib.INTEGRAL_STATE, "entropy": _lib.INTEGRAL_ENTROPY,
             "entropy_production": _lib.INTEGRAL_ENTROPY_PRODUCTION, "du": _lib.INTEGRAL_DU}
    _check_state(semi, u)
    if du is not None:
        _check_state(semi, du)
    out = np.zeros(max(8, semi.equations.nvariables))
    _lib.check(semi._lib.trixi_integrate(semi._handle, C.c_void_p(u.data_ptr()),
                                         C.c_void_p(du.data_ptr()) if du is not None else None, codes[which],
                                         out.ctypes.data_as(C.POINTER(C.c_double)), out.size,
                                         _stream_handle(stream)), semi._handle)
    n = semi.equations.nvariables if which in ("state", "du") else 1
    return out[:n].copy()


def calc_error_norms(u, semi, t=0.0, kind="convergence_test", params=None, u_ref=None, stream=None):
    """(L2, Linf) per variable on 2*polydeg+1 analysis nodes (reference
    calc_error_norms, src/callbacks_step/analysis_dg_2d.jl:44-89) against an
    analytic initial condition or a second state `u_ref`."""
    _check_state(semi, u)
    if u_ref is not None:
        _check_state(semi, u_ref)
    code, ptr, n, keep = _ic_args(kind, params)
    nv = semi.equations.nvariables
    l2 = np.zeros(nv)
    linf = np.zeros(nv)
    _lib.check(semi._lib.trixi_calc_error_norms(
        semi._handle, C.c_void_p(u.data_ptr()), C.c_void_p(u_ref.data_ptr()) if u_ref is not None else None, code,
        ptr, n, float(t), l2.ctypes.data_as(C.POINTER(C.c_double)), linf.ctypes.data_as(C.POINTER(C.c_double)),
        _stream_handle(stream)), semi._handle)
    return l2, linf


def synchronize(semi, stream=None):
    _call(semi, semi._lib.trixi_synchronize, stream=stream)
