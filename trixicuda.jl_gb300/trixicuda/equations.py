"""Equation systems, numerical-flux selectors and initial conditions.

The equation and flux names follow Trixi.jl's, which the reference uses
through `using Trixi` (src/TrixiCUDA.jl:12-55): LinearScalarAdvectionEquation
{1,2,3}D, CompressibleEulerEquations{1,2,3}D, flux, flux_ranocha, flux_central,
flux_lax_friedrichs.  The arithmetic itself runs in libtrixi_b200.so; these
objects only select it.  Initial conditions are evaluated on the host with
numpy (vectorised over nodes) and copied to the device once.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib


# --- numerical fluxes ---------------------------------------------------------
@dataclass(frozen=True)
class NumericalFlux:
    name: str
    code: int

    def __repr__(self) -> str:
        return self.name


flux_lax_friedrichs = NumericalFlux("flux_lax_friedrichs", _lib.FLUX_LAX_FRIEDRICHS)
flux_ranocha = NumericalFlux("flux_ranocha", _lib.FLUX_RANOCHA)
flux_central = NumericalFlux("flux_central", _lib.FLUX_CENTRAL)
flux_lax_friedrichs_naive = NumericalFlux("flux_lax_friedrichs_naive", _lib.FLUX_LAX_FRIEDRICHS_NAIVE)
flux = NumericalFlux("flux", -1)  # physical flux (weak form)
flux_hindenlang_gassner = NumericalFlux("flux_hindenlang_gassner", _lib.FLUX_HINDENLANG_GASSNER)
flux_shima_etal = NumericalFlux("flux_shima_etal", _lib.FLUX_SHIMA_ETAL)
flux_hll = NumericalFlux("flux_hll", _lib.FLUX_HLL)
flux_hlle = NumericalFlux("flux_hlle", _lib.FLUX_HLLE)


@dataclass(frozen=True)
class NonconservativeFlux:
    """The nonconservative half of a `(flux, nonconservative_flux)` pair, as
    Trixi's equations with nonconservative terms take them."""
    name: str
    code: int

    def __repr__(self) -> str:
        return self.name


flux_nonconservative_powell = NonconservativeFlux("flux_nonconservative_powell", _lib.NONCONSERVATIVE_POWELL)


def split_flux(f):
    """(symmetric flux, nonconservative flux or None) of a flux or a
    `(flux, nonconservative_flux)` tuple."""
    if isinstance(f, tuple):
        if len(f) != 2 or not isinstance(f[0], NumericalFlux) or not isinstance(f[1], NonconservativeFlux):
            raise ValueError(f"expected (flux, nonconservative_flux), got {f!r}")
        return f[0], f[1]
    return f, None


# --- equations ------------------------------------------------------------------
class AbstractEquations:
    ndims: int
    nvariables: int
    code: int

    def cons2prim(self, u):
        return u


class _LinearScalarAdvection(AbstractEquations):
    code = _lib.EQ_LINEAR_ADVECTION
    nvariables = 1

    def __init__(self, advection_velocity):
        a = np.atleast_1d(np.asarray(advection_velocity, dtype=np.float64))
        if a.shape != (self.ndims,):
            raise ValueError(f"advection velocity needs {self.ndims} components")
        self.advection_velocity = a
        self.gamma = 1.4

    def __repr__(self):
        return f"LinearScalarAdvectionEquation{self.ndims}D({tuple(self.advection_velocity)})"


class LinearScalarAdvectionEquation1D(_LinearScalarAdvection):
    ndims = 1


class LinearScalarAdvectionEquation2D(_LinearScalarAdvection):
    ndims = 2


class LinearScalarAdvectionEquation3D(_LinearScalarAdvection):
    ndims = 3


class _CompressibleEuler(AbstractEquations):
    code = _lib.EQ_COMPRESSIBLE_EULER

    def __init__(self, gamma: float = 1.4):
        self.gamma = float(gamma)
        self.nvariables = self.ndims + 2
        self.advection_velocity = np.zeros(self.ndims)

    def __repr__(self):
        return f"CompressibleEulerEquations{self.ndims}D({self.gamma})"

    def prim2cons(self, rho, v, p):
        """rho (n,), v (ndims, n), p (n,) -> u (nvars, n)."""
        rho = np.asarray(rho, dtype=np.float64)
        v = np.asarray(v, dtype=np.float64).reshape(self.ndims, -1)
        u = np.empty((self.nvariables,) + rho.shape)
        u[0] = rho
        u[1:1 + self.ndims] = rho * v
        u[-1] = p / (self.gamma - 1) + 0.5 * rho * np.sum(v * v, axis=0)
        return u

    def cons2prim(self, u):
        rho = u[0]
        v = u[1:1 + self.ndims] / rho
        p = (self.gamma - 1) * (u[-1] - 0.5 * np.sum(u[1:1 + self.ndims] * v, axis=0))
        return rho, v, p


class CompressibleEulerEquations1D(_CompressibleEuler):
    ndims = 1


class CompressibleEulerEquations2D(_CompressibleEuler):
    ndims = 2


class CompressibleEulerEquations3D(_CompressibleEuler):
    ndims = 3


class _IdealGlmMhd(AbstractEquations):
    """Ideal GLM-MHD (Trixi's IdealGlmMhdEquations{1,2,3}D): conservative
    variables (rho, rho v1, rho v2, rho v3, E, B1, B2, B3[, psi]) -- three
    velocity and field components in every dimension, the divergence-cleaning
    field psi in 2D and 3D, which have the nonconservative Powell terms.
    `c_h` is the GLM cleaning speed (a GlmSpeedCallback sets it during a run);
    it starts as NaN, as Trixi's `initial_c_h` default does."""
    code = _lib.EQ_IDEAL_GLM_MHD

    def __init__(self, gamma: float = 1.4, initial_c_h: float = float("nan")):
        self.gamma = float(gamma)
        self.c_h = float(initial_c_h)
        self.nvariables = 8 if self.ndims == 1 else 9
        self.advection_velocity = np.zeros(self.ndims)

    @property
    def have_nonconservative_terms(self) -> bool:
        return self.ndims > 1

    def __repr__(self):
        return f"IdealGlmMhdEquations{self.ndims}D({self.gamma}, c_h={self.c_h})"

    def prim2cons(self, rho, v, p, B=None, psi=None):
        """rho (n,), v (3, n), p (n,), B (3, n), psi (n,) -> u (nvars, n)."""
        rho = np.asarray(rho, dtype=np.float64)
        n = rho.shape
        v = np.asarray(v, dtype=np.float64).reshape((3,) + n)
        B = np.zeros((3,) + n) if B is None else np.asarray(B, dtype=np.float64).reshape((3,) + n)
        psi = np.zeros(n) if psi is None else np.asarray(psi, dtype=np.float64).reshape(n)
        u = np.empty((self.nvariables,) + n)
        u[0] = rho
        u[1:4] = rho * v
        u[4] = (p / (self.gamma - 1) + 0.5 * rho * np.sum(v * v, axis=0) + 0.5 * np.sum(B * B, axis=0))
        u[5:8] = B
        if self.nvariables == 9:
            u[4] += 0.5 * psi * psi
            u[8] = psi
        return u

    def cons2prim(self, u):
        """(rho, v (3, n), p): p = (gamma-1)(E - rho|v|^2/2 - |B|^2/2 - psi^2/2)."""
        rho = u[0]
        v = u[1:4] / rho
        psi2 = u[8] * u[8] if self.nvariables == 9 else 0.0
        p = (self.gamma - 1) * (u[4] - 0.5 * np.sum(u[1:4] * v, axis=0) - 0.5 * np.sum(u[5:8] * u[5:8], axis=0)
                                - 0.5 * psi2)
        return rho, v, p


class IdealGlmMhdEquations1D(_IdealGlmMhd):
    ndims = 1


class IdealGlmMhdEquations2D(_IdealGlmMhd):
    ndims = 2


class IdealGlmMhdEquations3D(_IdealGlmMhd):
    ndims = 3


# --- initial conditions (x: (ndims, n) array) -----------------------------------
def initial_condition_convergence_test(x, t, equations):
    """Advection: c + A sin(omega (sum(x) - t*sum(a)))... per dimension as in
    Trixi's linear-advection convergence test: u = 1 + 0.5 sin(pi * (x - a t))
    summed over dimensions with a 2-periodic domain."""
    x = np.atleast_2d(x)
    if isinstance(equations, _LinearScalarAdvection):
        c, A, L = 1.0, 0.5, 2.0
        omega = 2 * np.pi / L
        xt = x - equations.advection_velocity[:, None] * t
        return (c + A * np.sin(omega * np.sum(xt, axis=0)))[None, :]
    if isinstance(equations, _IdealGlmMhd):
        return _mhd_alfven_wave(x, t, equations)
    # Euler manufactured solution (source terms are not part of the hot path)
    c, A, L = 2.0, 0.1, 2.0
    omega = 2 * np.pi / L
    ini = c + A * np.sin(omega * (np.sum(x, axis=0) - t))
    rho = ini
    v = np.ones((equations.ndims,) + rho.shape)
    rho_e = ini * ini
    u = np.empty((equations.nvariables,) + rho.shape)
    u[0] = rho
    u[1:1 + equations.ndims] = rho * v
    u[-1] = rho_e
    return u


def _mhd_alfven_wave(x, t, eq):
    """Smooth circularly polarised Alfven waves, the convergence tests of
    ideal MHD.  1D and 2D: Derigs et al., "A novel high-order,
    entropy stable, 3D AMR MHD solver with guaranteed positive pressure",
    JCP 317 (2016) -- rho = 1, p = 0.1, unit background field along the
    propagation direction (the x axis in 1D; alpha = pi/4 in 2D on
    [0, sqrt 2]^2), perturbation amplitude 0.1, speed 1 (gamma = 5/3).
    3D: Altmann's thesis (2012) set-up on [-1, 1]^3 -- propagation along
    (1, 0, 2)/sqrt 5, amplitude 0.2, wave number 2 pi / 2 on the box."""
    n = x.shape[1]
    if eq.ndims == 1:
        arg = 2 * np.pi * (x[0] + t)
        v = np.stack([np.zeros(n), 0.1 * np.sin(arg), 0.1 * np.cos(arg)])
        B = np.stack([np.ones(n), v[1], v[2]])
        return eq.prim2cons(np.ones(n), v, np.full(n, 0.1), B)
    if eq.ndims == 2:
        alpha = 0.25 * np.pi
        x_perp = x[0] * np.cos(alpha) + x[1] * np.sin(alpha)
        b_perp = 0.1 * np.sin(2 * np.pi * (x_perp + t))
        v = np.stack([-b_perp * np.sin(alpha), b_perp * np.cos(alpha), 0.1 * np.cos(2 * np.pi * (x_perp + t))])
        B = np.stack([np.cos(alpha) + v[0], np.sin(alpha) + v[1], v[2]])
        return eq.prim2cons(np.ones(n), v, np.full(n, 0.1), B, np.zeros(n))
    omega, r, e = 2 * np.pi, 2.0, 0.2
    nx, ny = 1 / np.sqrt(r * r + 1), r / np.sqrt(r * r + 1)
    va = omega / ny
    ph = omega / ny * (nx * (x[0] - 0.5 * r) + ny * (x[2] - 0.5 * r)) - va * t
    v = np.stack([-e * ny * np.cos(ph), e * np.sin(ph), e * nx * np.cos(ph)])
    B = np.stack([nx - v[0], -v[1], ny - v[2]])
    return eq.prim2cons(np.ones(n), v, np.ones(n), B, np.zeros(n))


def initial_condition_constant(x, t, equations, rho=1.0, v=None, p=1.0):
    x = np.atleast_2d(x)
    n = x.shape[1]
    if isinstance(equations, _LinearScalarAdvection):
        return np.full((1, n), 1.0)
    if isinstance(equations, _IdealGlmMhd):
        v = np.zeros(3) if v is None else np.resize(np.asarray(v, dtype=np.float64), 3)
        return equations.prim2cons(np.full(n, rho), np.repeat(v[:, None], n, axis=1), np.full(n, p),
                                   np.ones((3, n)), np.zeros(n))
    v = np.zeros(equations.ndims) if v is None else np.asarray(v, dtype=np.float64)
    return equations.prim2cons(np.full(n, rho), np.repeat(v[:, None], n, axis=1), np.full(n, p))


def initial_condition_weak_blast_wave(x, t, equations):
    """Weak blast wave (Trixi's `initial_condition_weak_blast_wave`): inside
    r < 0.5 rho=1.1691, radial velocity 0.1882, p=1.245; outside rho=1, v=0, p=1."""
    x = np.atleast_2d(x)
    d = equations.ndims
    r = np.sqrt(np.sum(x * x, axis=0))
    rho = np.where(r > 0.5, 1.0, 1.1691)
    p = np.where(r > 0.5, 1.0, 1.245)
    v = np.zeros((d,) + r.shape)
    if d == 1:
        v[0] = np.where(r > 0.5, 0.0, 0.1882 * np.sign(x[0]))
    elif d == 2:
        phi = np.arctan2(x[1], x[0])
        v[0] = np.where(r > 0.5, 0.0, 0.1882 * np.cos(phi))
        v[1] = np.where(r > 0.5, 0.0, 0.1882 * np.sin(phi))
    else:
        phi = np.arctan2(x[1], x[0])
        theta = np.where(r == 0, 0.0, np.arccos(np.clip(x[2] / np.where(r == 0, 1.0, r), -1, 1)))
        v[0] = np.where(r > 0.5, 0.0, 0.1882 * np.cos(phi) * np.sin(theta))
        v[1] = np.where(r > 0.5, 0.0, 0.1882 * np.sin(phi) * np.sin(theta))
        v[2] = np.where(r > 0.5, 0.0, 0.1882 * np.cos(theta))
    if isinstance(equations, _IdealGlmMhd):
        # the MHD variant: the same jump, in a uniform field B = (1, 1, 1)
        v3 = np.zeros((3,) + r.shape)
        v3[:d] = v
        return equations.prim2cons(rho, v3, p, np.ones((3,) + r.shape), np.zeros(r.shape))
    return equations.prim2cons(rho, v, p)


class FourierField:
    """Seeded smooth periodic field: sum of random Fourier modes with integer
    wave vectors 0 < |k| <= kmax on the box [xmin, xmax]^d, scaled so that
    max |field| <= 1 (coefficients normalised by the sum of their magnitudes)."""

    def __init__(self, ndims, kmax, seed, xmin, xmax):
        rng = np.random.default_rng(seed)
        ks = [k for k in np.ndindex(*([2 * kmax + 1] * ndims))]
        ks = np.array(ks, dtype=np.int64) - kmax
        norm = np.sqrt(np.sum(ks * ks, axis=1))
        ks = ks[(norm > 0) & (norm <= kmax)]
        self.k = ks.astype(np.float64)
        a = rng.standard_normal(len(ks))
        b = rng.standard_normal(len(ks))
        s = np.sum(np.abs(a) + np.abs(b))
        self.a, self.b = a / s, b / s
        self.xmin = float(xmin)
        self.L = float(xmax) - float(xmin)

    def __call__(self, x):
        x = np.atleast_2d(x)
        phase = 2 * np.pi * (self.k @ (x - self.xmin)) / self.L  # (nk, n)
        return self.a @ np.cos(phase) + self.b @ np.sin(phase)


def initial_condition_fourier_euler(equations, seed=20261203, kmax=8, xmin=-2.0, xmax=2.0,
                                    amplitude=0.1, v0=(0.1, 0.2, 0.05), v_amp=0.02):
    """rho = 1 + amplitude * F_0(x), v = v0 + v_amp * F_{1..d}(x), p = 1 with
    independent seeded Fourier fields F (the synthetic 2D Euler workload)."""
    d = equations.ndims
    f_rho = FourierField(d, kmax, seed, xmin, xmax)
    f_v = [FourierField(d, kmax, seed + 1 + i, xmin, xmax) for i in range(d)]

    def ic(x, t, eq):
        x = np.atleast_2d(x)
        rho = 1.0 + amplitude * f_rho(x)
        v = np.stack([v0[i] + v_amp * f_v[i](x) for i in range(d)])
        p = np.ones_like(rho)
        return eq.prim2cons(rho, v, p)

    return ic


def initial_condition_fourier_advection(equations, seed=20261203, kmax=8, xmin=-2.0, xmax=2.0, amplitude=0.1):
    f = FourierField(equations.ndims, kmax, seed, xmin, xmax)

    def ic(x, t, eq):
        return (1.0 + amplitude * f(np.atleast_2d(x)))[None, :]

    return ic


# --- boundary conditions and source terms --------------------------------------
boundary_condition_periodic = "periodic"


class BoundaryConditionDirichlet:
    """Trixi's `BoundaryConditionDirichlet(boundary_value_function)`: the
    boundary value function's state at the face node and time t enters the
    surface flux as the outer state.  The library evaluates built-in
    functions on the device: initial_condition_convergence_test,
    initial_condition_constant, initial_condition_weak_blast_wave."""

    def __init__(self, boundary_value_function):
        self.boundary_value_function = boundary_value_function

    def __eq__(self, other):
        return (isinstance(other, BoundaryConditionDirichlet)
                and other.boundary_value_function is self.boundary_value_function)

    def __hash__(self):
        return hash(self.boundary_value_function)


def source_terms_convergence_test(u, x, t, equations):
    """Source of the Euler convergence test's manufactured solution
    rho = rho v_d = 2 + 0.1 sin(pi (sum_d x_d - t)), E = rho^2 (host version;
    the library evaluates it on the device).  x: (ndims, n)."""
    x = np.atleast_2d(x)
    d = equations.ndims
    g = equations.gamma
    c, A, L = 2.0, 0.1, 2.0
    omega = 2 * np.pi / L
    arg = omega * (np.sum(x, axis=0) - t)
    rho = c + A * np.sin(arg)
    rx = omega * A * np.cos(arg)
    s = np.empty((d + 2,) + rho.shape)
    if d == 1:
        s[0] = 0.0
        s[1] = s[2] = 0.5 * rx * (g - 1) * (4 * rho - 1)
    elif d == 2:
        s[0] = rx
        s[1] = s[2] = rx * (2 * g * rho - g - 2 * rho + 2)
        s[3] = 2 * rx * (2 * g * rho - g - rho + 1)
    else:
        s[0] = 2 * rx
        s[1] = s[2] = s[3] = 0.5 * rx * (4 * g * rho - 3 * g - 4 * rho + 7)
        s[4] = 0.5 * rx * (12 * g * rho - 9 * g - 4 * rho + 9)
    return s


def initial_condition_eoc_test_coupled_euler_gravity(x, t, equations):
    """The manufactured solution of the Euler-gravity convergence test
    (Schlottke-Lakemper, Winters, Ranocha, Gassner, JCP 442 (2021)):
    rho = 2 + 0.1 sin(pi (sum_d x_d - t)), v_d = 1 and the pressure of
    hydrostatic balance with the potential of rho (lap phi = 4 pi G rho,
    grad p = -rho grad phi), p = 2 G rho^2 / (ndims pi) with G = 1.  The
    reference's euler_convergence.jl (3D) runs it with gamma = 2.  x: (ndims, n)."""
    if not isinstance(equations, _CompressibleEuler):
        raise ValueError("the Euler-gravity convergence test needs the Euler equations")
    x = np.atleast_2d(x)
    d = equations.ndims
    rho = 2.0 + 0.1 * np.sin(np.pi * (np.sum(x, axis=0) - t))
    p = 2.0 * rho * rho / (d * np.pi)
    u = np.empty((d + 2,) + rho.shape)
    u[0] = rho
    u[1:1 + d] = rho
    u[-1] = p / (equations.gamma - 1) + 0.5 * rho * d
    return u


def source_terms_eoc_test_euler(u, x, t, equations):
    """Source that makes initial_condition_eoc_test_coupled_euler_gravity an
    exact solution of the Euler equations without gravity (host version; the
    library evaluates it on the device): with rx = 0.1 pi cos(pi (sum x - t))
    and K = 2/(ndims pi), mass (ndims-1) rx, momentum rx (ndims-1 + 2 K rho)
    per component, energy rx ((ndims-1)(2 K rho/(gamma-1) + ndims/2)
    + 2 ndims K rho).  x: (ndims, n)."""
    x = np.atleast_2d(x)
    d = equations.ndims
    g = equations.gamma
    arg = np.pi * (np.sum(x, axis=0) - t)
    rho = 2.0 + 0.1 * np.sin(arg)
    rx = 0.1 * np.pi * np.cos(arg)
    kr2 = 2.0 * (2.0 / (d * np.pi)) * rho
    s = np.empty((d + 2,) + rho.shape)
    s[0] = (d - 1) * rx
    s[1:1 + d] = rx * ((d - 1) + kr2)
    s[-1] = rx * ((d - 1) * (kr2 / (g - 1) + 0.5 * d) + d * kr2)
    return s


def boundary_function_code(func):
    """trixi_initial_condition_kind of a built-in boundary value function."""
    codes = {initial_condition_constant: _lib.IC_CONSTANT,
             initial_condition_convergence_test: _lib.IC_CONVERGENCE_TEST,
             initial_condition_weak_blast_wave: _lib.IC_WEAK_BLAST_WAVE,
             initial_condition_eoc_test_coupled_euler_gravity: _lib.IC_EOC_TEST_COUPLED_EULER_GRAVITY}
    if func not in codes:
        raise NotImplementedError("Dirichlet boundary values: the built-in initial conditions only")
    return codes[func]
