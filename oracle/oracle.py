"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY -- the checker for libtrixi_b200.so.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
Parity status: unpinned at the Trixi.jl boundary (see trixi_oracle.c).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import build as _build_mod

EQ_ADVECTION, EQ_EULER, EQ_MHD = 0, 1, 2
VOL_WEAK, VOL_FLUXDIFF, VOL_SHOCK_HG = 0, 1, 2
FLUX_LLF, FLUX_RANOCHA, FLUX_CENTRAL, FLUX_LLF_NAIVE, FLUX_HINDENLANG_GASSNER = 0, 1, 2, 3, 4
FLUX_SHIMA_ETAL, FLUX_HLL, FLUX_HLLE = 5, 6, 7
NONCONS_NONE, NONCONS_POWELL = 0, 1


class OracleDesc(C.Structure):
    _fields_ = [
        ("ndims", C.c_int32), ("polydeg", C.c_int32), ("nvars", C.c_int32), ("equation", C.c_int32),
        ("gamma", C.c_double), ("advection_velocity", C.c_double * 3),
        ("volume_integral", C.c_int32), ("volume_flux", C.c_int32), ("surface_flux", C.c_int32),
        ("volume_flux_fv", C.c_int32),
        ("alpha_max", C.c_double), ("alpha_min", C.c_double), ("alpha_smooth", C.c_int32),
        ("nelements", C.c_int64), ("ninterfaces", C.c_int64), ("nmortars", C.c_int64),
        ("inverse_jacobian", C.POINTER(C.c_double)),
        ("interface_neighbor_ids", C.POINTER(C.c_int64)), ("interface_orientations", C.POINTER(C.c_int64)),
        ("mortar_neighbor_ids", C.POINTER(C.c_int64)), ("mortar_large_sides", C.POINTER(C.c_int64)),
        ("mortar_orientations", C.POINTER(C.c_int64)),
        ("nboundaries", C.c_int64),
        ("boundary_neighbor_ids", C.POINTER(C.c_int64)), ("boundary_neighbor_sides", C.POINTER(C.c_int64)),
        ("boundary_orientations", C.POINTER(C.c_int64)),
        ("boundary_function", C.c_int32), ("source_terms", C.c_int32),
        ("boundary_params", C.c_double * 8), ("source_params", C.c_double * 3),
        ("node_coordinates", C.POINTER(C.c_double)),
        ("nonconservative_flux", C.c_int32), ("glm_speed", C.c_double),
        ("indicator_variable", C.c_int32),
    ]


_lib = None
_PD = C.POINTER(C.c_double)


def load():
    global _lib
    if _lib is None:
        path = _build_mod.build()
        lib = C.CDLL(str(path))
        lib.oracle_basis.restype = C.c_int
        lib.oracle_basis.argtypes = [C.c_int] + [_PD] * 10
        lib.oracle_create.restype = C.c_void_p
        lib.oracle_create.argtypes = [C.POINTER(OracleDesc)]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        lib.oracle_set_threads.restype = C.c_int
        lib.oracle_set_threads.argtypes = [C.c_int]
        for name, args in [
            ("oracle_volume_integral", [C.c_void_p, _PD, _PD, _PD]),
            ("oracle_prolong2interfaces", [C.c_void_p, _PD, _PD]),
            ("oracle_interface_flux", [C.c_void_p, _PD, _PD]),
            ("oracle_prolong2mortars", [C.c_void_p, _PD, C.POINTER(_PD)]),
            ("oracle_mortar_flux", [C.c_void_p, C.POINTER(_PD), _PD]),
            ("oracle_surface_integral", [C.c_void_p, _PD, _PD]),
            ("oracle_jacobian", [C.c_void_p, _PD]),
            ("oracle_indicator_hg", [C.c_void_p, _PD, _PD]),
            ("oracle_rhs", [C.c_void_p, _PD, _PD, C.c_double]),
            ("oracle_rk_ck2n54", [C.c_void_p, _PD, _PD, C.c_double, C.c_double, C.c_int]),
            ("oracle_prolong2boundaries", [C.c_void_p, _PD, _PD]),
            ("oracle_boundary_flux", [C.c_void_p, _PD, C.c_double, _PD]),
            ("oracle_sources", [C.c_void_p, _PD, C.c_double]),
            ("oracle_eval_ic", [C.c_void_p, C.c_int, _PD, _PD, C.c_double, _PD]),
            ("oracle_physical_flux", [C.c_void_p, _PD, C.c_int, _PD]),
            ("oracle_two_point_flux", [C.c_void_p, C.c_int, _PD, _PD, C.c_int, _PD]),
            ("oracle_noncons_flux", [C.c_void_p, _PD, _PD, C.c_int, _PD]),
        ]:
            fn = getattr(lib, name)
            fn.restype = None
            fn.argtypes = args
        lib.oracle_size.restype = C.c_int64
        lib.oracle_size.argtypes = [C.c_void_p, C.c_int]
        _lib = lib
    return _lib


def _pd(a):
    return a.ctypes.data_as(_PD)


def basis(polydeg: int) -> dict:
    n = polydeg + 1
    out = {k: np.zeros(n if k in ("nodes", "weights") else n * n) for k in
           ("nodes", "weights", "dmat", "dsplit", "dhat", "ivdm", "fup", "flo", "rup", "rlo")}
    st = load().oracle_basis(polydeg, *[_pd(out[k]) for k in
                                        ("nodes", "weights", "dmat", "dsplit", "dhat", "ivdm", "fup", "flo", "rup", "rlo")])
    if st != 0:
        raise ValueError(f"oracle_basis({polydeg}) failed: {st}")
    for k in out:
        if out[k].size == n * n:
            out[k] = out[k].reshape(n, n, order="F")
    return out


class Oracle:
    """CPU restatement of the semidiscretization for one problem."""

    def __init__(self, containers, ndims, polydeg, nvars, equation, gamma=1.4, advection_velocity=(0, 0, 0),
                 volume_integral=VOL_WEAK, volume_flux=FLUX_CENTRAL, surface_flux=FLUX_LLF,
                 volume_flux_fv=FLUX_LLF, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True,
                 boundary_function=-1, boundary_params=None, source_terms=0, source_params=None,
                 nonconservative_flux=NONCONS_NONE, glm_speed=0.0, indicator_variable=0):
        lib = load()
        self._keep = dict(
            inv=np.ascontiguousarray(containers.inverse_jacobian, dtype=np.float64),
            if_nid=np.ascontiguousarray(containers.interface_neighbor_ids, dtype=np.int64),
            if_ori=np.ascontiguousarray(containers.interface_orientations, dtype=np.int64),
            mo_nid=np.ascontiguousarray(containers.mortar_neighbor_ids, dtype=np.int64),
            mo_ls=np.ascontiguousarray(containers.mortar_large_sides, dtype=np.int64),
            mo_ori=np.ascontiguousarray(containers.mortar_orientations, dtype=np.int64),
            b_nid=np.ascontiguousarray(containers.boundary_neighbor_ids, dtype=np.int64),
            b_side=np.ascontiguousarray(containers.boundary_neighbor_sides, dtype=np.int64),
            b_ori=np.ascontiguousarray(containers.boundary_orientations, dtype=np.int64),
            coords=np.ascontiguousarray(containers.node_coordinates, dtype=np.float64),
        )
        k = self._keep
        d = OracleDesc()
        d.ndims, d.polydeg, d.nvars, d.equation = ndims, polydeg, nvars, equation
        d.gamma = gamma
        av = list(advection_velocity) + [0.0] * (3 - len(advection_velocity))
        for i in range(3):
            d.advection_velocity[i] = av[i]
        d.volume_integral, d.volume_flux, d.surface_flux, d.volume_flux_fv = (
            volume_integral, volume_flux, surface_flux, volume_flux_fv)
        d.alpha_max, d.alpha_min, d.alpha_smooth = alpha_max, alpha_min, int(alpha_smooth)
        d.nelements = containers.nelements
        d.ninterfaces = containers.ninterfaces
        d.nmortars = containers.nmortars
        d.inverse_jacobian = _pd(k["inv"])
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))  # noqa: E731
        d.interface_neighbor_ids, d.interface_orientations = ip(k["if_nid"]), ip(k["if_ori"])
        d.mortar_neighbor_ids, d.mortar_large_sides, d.mortar_orientations = ip(k["mo_nid"]), ip(k["mo_ls"]), ip(k["mo_ori"])
        d.nboundaries = containers.nboundaries
        d.boundary_neighbor_ids, d.boundary_neighbor_sides = ip(k["b_nid"]), ip(k["b_side"])
        d.boundary_orientations = ip(k["b_ori"])
        d.boundary_function, d.source_terms = int(boundary_function), int(source_terms)
        for i, v in enumerate(boundary_params if boundary_params is not None else []):
            d.boundary_params[i] = float(v)
        for i, v in enumerate(source_params if source_params is not None else (2.0, 0.1, 2.0)):
            d.source_params[i] = float(v)
        d.node_coordinates = _pd(k["coords"])
        d.nonconservative_flux, d.glm_speed = int(nonconservative_flux), float(glm_speed)
        d.indicator_variable = int(indicator_variable)
        self._desc = d
        self._h = lib.oracle_create(C.byref(d))
        if not self._h:
            raise ValueError("oracle_create failed")
        self.lib = lib
        self.ndims, self.N, self.nv = ndims, polydeg + 1, nvars
        self.nelements = containers.nelements
        self.nchild = 2 ** (ndims - 1)

    @staticmethod
    def own_containers(mesh, polydeg):
        """The oracle's own connectivity for a TreeMesh's parameters (domain,
        level, refinement boxes, periodicity), built by oracle/treemesh.py
        with the oracle's LGL nodes -- no product code involved."""
        from .treemesh import OracleTreeMesh

        tm = OracleTreeMesh(mesh.coordinates_min, mesh.coordinates_max, mesh.initial_refinement_level,
                            getattr(mesh, "refinement_patches", ()), getattr(mesh, "periodicity", True))
        return tm.containers(basis(polydeg)["nodes"])

    @classmethod
    def from_semi(cls, semi):
        """Oracle for the same problem as a SemidiscretizationHyperbolicGPU.
        When the semi carries its TreeMesh, the oracle computes on its own
        connectivity (own_containers); a semi that only carries containers
        (a partition's local mesh with ghosts) is taken as given."""
        from trixicuda.semidiscretization import flux_codes
        from trixicuda.solver import VolumeIntegralShockCapturingHG

        eq, sol = semi.equations, semi.solver
        vi = sol.volume_integral
        codes = flux_codes(sol, eq)
        kw = dict(volume_integral=vi.code, surface_flux=codes["surface_flux"], volume_flux=codes["volume_flux"],
                  volume_flux_fv=codes["volume_flux_fv"], nonconservative_flux=codes["nonconservative_flux"],
                  glm_speed=float(getattr(eq, "c_h", 0.0)))
        if isinstance(vi, VolumeIntegralShockCapturingHG):
            kw.update(alpha_max=vi.indicator.alpha_max, alpha_min=vi.indicator.alpha_min,
                      alpha_smooth=vi.indicator.alpha_smooth, indicator_variable=vi.indicator.variable_code)
        av = tuple(getattr(eq, "advection_velocity", np.zeros(eq.ndims)))
        # boundary function and source terms, with the library's parameters
        d = getattr(semi, "_desc", None)
        if d is not None and d.nboundaries > 0:
            code = int(d.boundary_function)
            if code == 1:  # convergence test defaults (advection: 1, 0.5, 2; Euler: 2, 0.1, 2)
                params = (1.0, 0.5, 2.0) if eq.nvariables == 1 else (2.0, 0.1, 2.0)
            else:
                params = [d.boundary_params[i] for i in range(8)]
            if d.nboundary_params > 0:
                params = [d.boundary_params[i] for i in range(8)]
            kw.update(boundary_function=code, boundary_params=params)
        if d is not None and d.source_terms:
            kw.update(source_terms=int(d.source_terms))
        mesh = getattr(semi, "mesh", None)
        cont = cls.own_containers(mesh, sol.polydeg) if hasattr(mesh, "initial_refinement_level") else semi.containers
        return cls(cont, eq.ndims, sol.polydeg, eq.nvariables, eq.code,
                   gamma=getattr(eq, "gamma", 1.4), advection_velocity=av, **kw)

    def __del__(self):
        if getattr(self, "_h", None):
            self.lib.oracle_destroy(self._h)
            self._h = None

    # arrays are numpy float64 in reference memory layout (any shape, C-contiguous)
    def rhs(self, u: np.ndarray, t: float = 0.0) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        self.lib.oracle_rhs(self._h, _pd(du), _pd(u), float(t))
        return du

    def volume_integral(self, u, alpha=None):
        u = np.ascontiguousarray(u, dtype=np.float64)
        du = np.empty_like(u)
        a = np.zeros(self.nelements) if alpha is None else np.ascontiguousarray(alpha, dtype=np.float64)
        self.lib.oracle_volume_integral(self._h, _pd(du), _pd(u), _pd(a))
        return du

    def indicator(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        a = np.empty(self.nelements)
        self.lib.oracle_indicator_hg(self._h, _pd(u), _pd(a))
        return a

    def prolong2interfaces(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        iu = np.zeros(self.lib.oracle_size(self._h, 1))
        self.lib.oracle_prolong2interfaces(self._h, _pd(u), _pd(iu))
        return iu

    def interface_flux(self, iu, sfv=None):
        sfv = np.zeros(self.lib.oracle_size(self._h, 2)) if sfv is None else sfv
        self.lib.oracle_interface_flux(self._h, _pd(np.ascontiguousarray(iu)), _pd(sfv))
        return sfv

    def prolong2boundaries(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        bu = np.zeros(max(self.lib.oracle_size(self._h, 5), 1))
        self.lib.oracle_prolong2boundaries(self._h, _pd(u), _pd(bu))
        return bu

    def boundary_flux(self, bu, t, sfv):
        self.lib.oracle_boundary_flux(self._h, _pd(np.ascontiguousarray(bu)), float(t), _pd(sfv))
        return sfv

    def sources(self, du, t):
        self.lib.oracle_sources(self._h, _pd(du), float(t))
        return du

    def prolong2mortars(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        n = self.lib.oracle_size(self._h, 3)
        arrs = [np.zeros(max(n, 1)) for _ in range(self.nchild)]
        ptrs = (_PD * self.nchild)(*[_pd(a) for a in arrs])
        self.lib.oracle_prolong2mortars(self._h, _pd(u), ptrs)
        return arrs

    def mortar_flux(self, arrs, sfv):
        ptrs = (_PD * self.nchild)(*[_pd(a) for a in arrs])
        self.lib.oracle_mortar_flux(self._h, ptrs, _pd(sfv))
        return sfv

    def surface_integral(self, du, sfv):
        du = np.array(du, dtype=np.float64, copy=True)
        self.lib.oracle_surface_integral(self._h, _pd(du), _pd(np.ascontiguousarray(sfv)))
        return du

    def jacobian(self, du):
        du = np.array(du, dtype=np.float64, copy=True)
        self.lib.oracle_jacobian(self._h, _pd(du))
        return du

    # pointwise fluxes (u: nvars values)
    def physical_flux(self, u, o):
        u = np.ascontiguousarray(u, dtype=np.float64)
        f = np.zeros(self.nv)
        self.lib.oracle_physical_flux(self._h, _pd(u), int(o), _pd(f))
        return f

    def two_point_flux(self, kind, ul, ur, o):
        ul, ur = (np.ascontiguousarray(x, dtype=np.float64) for x in (ul, ur))
        f = np.zeros(self.nv)
        self.lib.oracle_two_point_flux(self._h, int(kind), _pd(ul), _pd(ur), int(o), _pd(f))
        return f

    def noncons_flux(self, ul, ur, o):
        ul, ur = (np.ascontiguousarray(x, dtype=np.float64) for x in (ul, ur))
        f = np.zeros(self.nv)
        self.lib.oracle_noncons_flux(self._h, _pd(ul), _pd(ur), int(o), _pd(f))
        return f

    def rk_ck2n54(self, u, t, dt, nsteps, k=None):
        u = np.array(u, dtype=np.float64, copy=True)
        k = np.zeros_like(u) if k is None else np.array(k, dtype=np.float64, copy=True)
        self.lib.oracle_rk_ck2n54(self._h, _pd(u), _pd(k), float(t), float(dt), int(nsteps))
        return u, k


def set_threads(n: int) -> int:
    return load().oracle_set_threads(int(n))


def default_threads() -> int:
    return os.cpu_count() or 1
