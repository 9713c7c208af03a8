"""DGSEMGPU solver description (reference: src/solvers/dgsem_gpu.jl:43-53).

`DGSEMGPU(polydeg=..., surface_flux=..., volume_integral=...)` records the
choices that the reference turns into a `DG{...}` with a GPU basis; here they
become the enum fields of the C ABI's trixi_problem_desc.  The LGL basis and
L2 mortar operators are computed by libtrixi_b200.so (trixi_lgl_basis), the
GB300 replacement of LobattoLegendreBasisGPU / MortarL2GPU
(src/solvers/basis_lobatto_legendre.jl:60-100, 155-173).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .equations import NumericalFlux, flux, flux_central, flux_lax_friedrichs


@dataclass
class VolumeIntegralWeakForm:
    code: int = _lib.VOLUME_WEAK_FORM


@dataclass
class VolumeIntegralFluxDifferencing:
    volume_flux: NumericalFlux = flux_central
    code: int = _lib.VOLUME_FLUX_DIFFERENCING


def density_pressure(u, equations):
    rho, _, p = equations.cons2prim(u)
    return rho * p


def pressure(u, equations):
    return equations.cons2prim(u)[2]


# indicator variables the library evaluates (trixi_problem_desc.indicator_variable)
INDICATOR_VARIABLES = {density_pressure: 0, pressure: 1}


@dataclass
class IndicatorHennemannGassner:
    """Hennemann-Gassner shock indicator (Trixi's IndicatorHennemannGassner,
    wrapped by the reference at src/solvers/indicators.jl:7-42)."""
    equations: object = None
    basis: object = None
    alpha_max: float = 0.5
    alpha_min: float = 0.001
    alpha_smooth: bool = True
    variable: object = density_pressure

    def __post_init__(self):
        if self.variable not in INDICATOR_VARIABLES:
            raise NotImplementedError("indicator variable: density_pressure or pressure")

    @property
    def variable_code(self) -> int:
        return INDICATOR_VARIABLES[self.variable]


@dataclass
class VolumeIntegralShockCapturingHG:
    indicator: IndicatorHennemannGassner
    volume_flux_dg: NumericalFlux = flux_central
    volume_flux_fv: NumericalFlux = flux_lax_friedrichs
    code: int = _lib.VOLUME_SHOCK_CAPTURING_HG


def lgl_basis_item(polydeg: int, name: str) -> np.ndarray:
    """An operator of the LGL basis from libtrixi_b200.so (host code, no GPU)."""
    n = polydeg + 1
    size = n if name in ("nodes", "weights") else n * n
    out = np.zeros(size, dtype=np.float64)
    st = _lib.load().trixi_lgl_basis(polydeg, _lib.BASIS_ITEMS[name],
                                     out.ctypes.data_as(C.POINTER(C.c_double)), size)
    _lib.check(st)
    if size == n:
        return out
    return out.reshape(n, n, order="F")  # Julia column-major matrix


class LobattoLegendreBasisGPU:
    """Nodal Lobatto-Legendre basis of degree `polydeg`."""

    def __init__(self, polydeg: int, RealT=np.float64):
        self.polydeg = int(polydeg)
        self.RealT = RealT
        self.nodes = lgl_basis_item(self.polydeg, "nodes")
        self.weights = lgl_basis_item(self.polydeg, "weights")
        self.inverse_weights = 1.0 / self.weights

    def nnodes(self) -> int:
        return self.polydeg + 1

    def matrix(self, name: str) -> np.ndarray:
        return lgl_basis_item(self.polydeg, name)


@dataclass
class DGSEMGPU:
    polydeg: int
    surface_flux: NumericalFlux = flux_central
    volume_integral: object = field(default_factory=VolumeIntegralWeakForm)
    RealT: object = np.float64

    def __post_init__(self):
        self.basis = LobattoLegendreBasisGPU(self.polydeg, self.RealT)
        if self.surface_flux is flux:
            raise ValueError("the physical flux is not a surface flux")

    def nnodes(self) -> int:
        return self.polydeg + 1
