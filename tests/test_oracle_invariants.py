"""Discrete invariants that pin the oracle without a live Trixi.jl:
free-stream preservation, conservation, entropy conservation of flux_ranocha,
the convergence order of the C1 advection problem, and the 2N-RK order."""
import numpy as np
import pytest

from problems import host_problem


def _const_state(s, u):
    eq = s.equations
    if eq.nvariables == 1:
        return np.full_like(u, 1.7)
    n = u.size // eq.nvariables
    rho = np.full(n, 1.3)
    v = np.tile(np.array([0.3, -0.2, 0.1])[: eq.ndims, None], (1, n))
    p = np.full(n, 0.9)
    return np.ascontiguousarray(eq.prim2cons(rho, v, p).T.reshape(u.shape))


CASES = [("adv_weak", 1, 3, False), ("adv_weak", 2, 2, True), ("adv_weak", 3, 1, True),
         ("euler_fd", 2, 2, False), ("euler_fd", 2, 2, True), ("euler_fd", 3, 1, True),
         ("euler_weak", 2, 2, True), ("euler_sc", 2, 2, True), ("euler_sc", 3, 1, False)]


@pytest.mark.parametrize("kind,d,level,refined", CASES)
def test_free_stream_preservation(kind, d, level, refined):
    s, orc, u = host_problem(kind, d, level, polydeg=3, refined=refined)
    u0 = _const_state(s, u)
    du = orc.rhs(u0)
    assert np.max(np.abs(du)) < 1e-11 * max(1.0, float(np.max(np.abs(s.containers.inverse_jacobian))))


def _mass(s, du):
    """sum_e J_e sum_i w_i du_i per variable (J = (1/invJ)^d)."""
    c = s.containers
    d = s.mesh.ndims
    w = s.solver.basis.weights
    W = w
    for _ in range(d - 1):
        W = np.multiply.outer(W, w)
    W = W.T.reshape(-1)  # memory order (z, y, x)
    J = (1.0 / c.inverse_jacobian) ** d
    nv = du.shape[-1]
    return np.einsum("env,n,e->v", du.reshape(c.nelements, -1, nv), W, J)


@pytest.mark.parametrize("kind,d,level,refined", CASES)
def test_conservation(kind, d, level, refined):
    s, orc, u = host_problem(kind, d, level, polydeg=3, refined=refined)
    du = orc.rhs(u)
    m = _mass(s, du)
    scale = np.max(np.abs(du)) * np.sum((1.0 / s.containers.inverse_jacobian) ** d)
    assert np.max(np.abs(m)) < 1e-12 * scale


@pytest.mark.parametrize("d,refined", [(2, False), (3, False)])
def test_entropy_conservation_flux_ranocha(d, refined):
    """flux_ranocha in the volume and on interfaces conserves the total
    entropy: sum J w v(u) . du = 0 with v the entropy variables."""
    s, orc, u = host_problem("euler_fd", d, 2 if d == 2 else 1, polydeg=3, refined=refined)
    du = orc.rhs(u)
    eq = s.equations
    g = eq.gamma
    uu = u.reshape(-1, eq.nvariables).T
    rho, v, p = eq.cons2prim(uu)
    srho = np.log(p) - g * np.log(rho)
    ent = np.empty_like(uu)
    v2 = np.sum(v * v, axis=0)
    ent[0] = (g - srho) / (g - 1) - 0.5 * rho * v2 / p
    ent[1:1 + d] = rho * v / p
    ent[-1] = -rho / p
    c = s.containers
    w = s.solver.basis.weights
    W = w
    for _ in range(d - 1):
        W = np.multiply.outer(W, w)
    W = np.broadcast_to(W.T[None], (c.nelements,) + W.shape).reshape(-1)
    J = np.repeat((1.0 / c.inverse_jacobian) ** d, (s.solver.polydeg + 1) ** d)
    dS = np.sum(W * J * np.sum(ent * du.reshape(-1, eq.nvariables).T, axis=0))
    scale = np.sum(W * J * np.sum(np.abs(ent * du.reshape(-1, eq.nvariables).T), axis=0))
    assert abs(dS) < 1e-11 * scale


def test_c1_advection_convergence_order():
    """C1 (1D advection, weak form, LLF, polydeg 3): the L2 error after t=1
    converges at order ~ N = polydeg + 1."""
    import trixicuda as T

    errs = []
    for level in (2, 3, 4):
        s, orc, u = host_problem("adv_weak", 1, level, polydeg=3)
        h = 2.0 / 2**level
        dt = 1.6 * h / 4 / 4   # CFL-limited, small enough for the time error to be negligible
        nsteps = int(round(1.0 / dt))
        dt = 1.0 / nsteps
        uT, _ = orc.rk_ck2n54(u, 0.0, dt, nsteps)
        x = s.containers.node_coordinates.reshape(-1)
        exact = 1 + 0.5 * np.sin(np.pi * (x - 1.0))
        w = np.tile(s.solver.basis.weights, s.containers.nelements) * h / 2
        errs.append(np.sqrt(np.sum(w * (uT.reshape(-1) - exact) ** 2)))
    eoc = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(eoc > 3.5), eoc


def test_rk_order_linear_ode():
    """The CK2N54 coefficients integrate y' = lambda y with 4th-order accuracy."""
    from trixicuda.time_integration import CK2N54_A, CK2N54_B

    def step(y, h, lam):
        k = 0.0
        for a, b in zip(CK2N54_A, CK2N54_B):
            k = a * k + h * lam * y
            y = y + b * k
        return y

    lam = -1.3 + 0.7j
    errs = []
    for n in (10, 20, 40):
        h = 1.0 / n
        y = 1.0
        for _ in range(n):
            y = step(y, h, lam)
        errs.append(abs(y - np.exp(lam)))
    eoc = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(eoc > 3.8), eoc
