"""Time integration: CarpenterKennedy2N54 with the RK stage fused into the
rhs kernel (the reference's examples use OrdinaryDiffEq's
`CarpenterKennedy2N54(williamson_condition = false)`,
examples/advection_basic_1d.jl:55, whose broadcast stage update runs outside
TrixiCUDA.jl).  Coefficients: Carpenter & Kennedy (1994), NASA TM-109112,
five-stage fourth-order 2N-storage scheme:
    k <- A_s k + dt f(u, t + c_s dt);   u <- u + B_s k.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import semidiscretization as sd

CK2N54_A = (0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
            -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0)
CK2N54_B = (1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
            1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
            2277821191437.0 / 14882151754819.0)
CK2N54_C = (0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
            2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0)


@dataclass
class CarpenterKennedy2N54:
    williamson_condition: bool = False


@dataclass
class ODESolution:
    u: object
    t: float
    nsteps: int


def solve(ode: sd.ODEProblem, alg=None, dt: float = None, nsteps: int | None = None, stream=None):
    """Integrates `ode` from tspan[0] to tspan[1] with fixed steps of size dt
    (the last step is shortened to hit tspan[1]).  All stages run on the GPU."""
    torch = sd._torch()
    semi = ode.p
    t0, t1 = ode.tspan
    if dt is None:
        raise ValueError("dt is required")
    u = ode.u0.clone()
    k = torch.zeros_like(u)
    n_full = int((t1 - t0) // dt) if nsteps is None else int(nsteps)
    t = t0
    if n_full > 0:
        sd.rk_steps(u, k, t, dt, n_full, semi, stream=stream)
        t = t0 + n_full * dt
    if nsteps is None and t1 - t > 1e-14 * max(1.0, abs(t1)):
        sd.rk_steps(u, k, t, t1 - t, 1, semi, stream=stream)
        t = t1
        n_full += 1
    return ODESolution(u, t, n_full)
