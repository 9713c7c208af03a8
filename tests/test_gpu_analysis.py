"""GPU versions of the reference's callback loops and initial-condition
kernel (max_dt, integrals, calc_error_norms, compute_coefficients), checked
against host restatements; plus size-independent invariants at the full
benchmark sizes: conservation of the quadrature integral of u over RK steps,
and zero entropy production of flux_ranocha flux differencing."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from problems import make, semi_and_oracle

pytestmark = pytest.mark.gpu


def _host_state(semi, u):
    return u.cpu().numpy().reshape(-1, semi.equations.nvariables).T


def test_compute_coefficients_gpu_matches_host(cuda):
    for kind, d, lvl, ic in [("adv_weak", 1, 4, "convergence_test"), ("adv_weak", 2, 3, "convergence_test"),
                             ("adv_weak", 3, 2, "convergence_test"), ("euler_sc", 2, 3, "weak_blast_wave"),
                             ("euler_sc", 3, 2, "weak_blast_wave")]:
        semi, _ = semi_and_oracle(kind, d, lvl)
        u = T.compute_coefficients_gpu(semi, ic)
        T.synchronize(semi)
        host = semi.compute_coefficients_host(0.0, {"convergence_test": T.initial_condition_convergence_test,
                                                    "weak_blast_wave": T.initial_condition_weak_blast_wave}[ic])
        np.testing.assert_allclose(u.cpu().numpy(), host, rtol=1e-14, atol=1e-14)


def test_max_dt_matches_host(cuda):
    for kind, d, lvl in [("euler_fd", 2, 3), ("euler_sc", 3, 2), ("adv_weak", 2, 3)]:
        semi, _ = semi_and_oracle(kind, d, lvl)
        u = semi.compute_coefficients()
        dt = T.max_dt(u, semi)
        eq = semi.equations
        uu = _host_state(semi, u)
        E = semi.nelements
        NN = semi.nnodes ** d
        if hasattr(eq, "cons2prim") and eq.nvariables > 1:
            rho, v, p = eq.cons2prim(uu)
            c = np.sqrt(eq.gamma * p / rho)
            lam = (np.abs(v) + c).reshape(d, E, NN).max(axis=2)
        else:
            lam = np.repeat(np.abs(eq.advection_velocity)[:, None], E, axis=1)
        scaled = semi.containers.inverse_jacobian * lam.sum(axis=0)
        ref = 2.0 / (semi.nnodes * scaled.max())
        assert abs(dt - ref) <= 1e-14 * ref


def _weights(semi):
    d = semi.mesh.ndims
    w = semi.solver.basis.weights
    W = w
    for _ in range(d - 1):
        W = np.multiply.outer(W, w)
    return W.T.reshape(-1)


def test_integrals_match_host(cuda):
    semi, orc = semi_and_oracle("euler_fd", 2, 3)
    u = semi.compute_coefficients()
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    tot = T.integrate(u, semi, "state")
    uu = u.cpu().numpy().reshape(semi.nelements, -1, 4)
    J = (1.0 / semi.containers.inverse_jacobian) ** 2
    ref = np.einsum("env,n,e->v", uu, _weights(semi), J)
    np.testing.assert_allclose(tot, ref, rtol=1e-13)
    mass_rate = T.integrate(u, semi, "du", du=du)
    assert np.max(np.abs(mass_rate)) < 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_full_size_c2_conservation_and_entropy(precision, cuda):
    """2D Euler level 7 (the benchmark size): flux_ranocha volume + surface
    conserves mass/momentum/energy and produces no entropy (to round-off)."""
    mesh, eq, _, solver, _ = make("euler_fd", 2, 7)
    ic = T.initial_condition_fourier_euler(eq, seed=20261203, kmax=8)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    u = semi.compute_coefficients()
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    s0 = T.integrate(u, semi, "state")
    prod = T.integrate(u, semi, "entropy_production", du=du)[0]
    scale = T.integrate(u, semi, "entropy")[0]
    dt = 0.5 * T.max_dt(u, semi)
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.0, dt, 5, semi)
    s1 = T.integrate(u, semi, "state")
    tol = 1e-13 if precision == "fp64" else 1e-9
    assert np.max(np.abs(s1 - s0) / np.abs(s0)) < tol
    if precision == "fp64":
        # entropy production relative to the entropy rate magnitude
        absprod = abs(prod)
        assert absprod < 1e-10 * abs(scale), (prod, scale)


def test_full_size_c3_conservation(cuda):
    """3D Euler shock capturing at level 5 (32768 elements): the DG-FV blend
    is conservative too."""
    mesh, eq, ic, solver, _ = make("euler_sc", 3, 5)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver)
    u = T.compute_coefficients_gpu(semi, "weak_blast_wave")
    s0 = T.integrate(u, semi, "state")
    dt = 0.5 * T.max_dt(u, semi)
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.0, dt, 3, semi)
    s1 = T.integrate(u, semi, "state")
    scale = np.abs(s0).max()
    assert np.max(np.abs(s1 - s0)) < 1e-13 * scale


def test_error_norms(cuda):
    """calc_error_norms: zero for the exact state, equals a host evaluation on
    analysis nodes for the advection convergence test, and mixed-vs-FP64
    distances through u_ref."""
    semi, orc = semi_and_oracle("adv_weak", 2, 3)
    u = T.compute_coefficients_gpu(semi, "convergence_test")
    l2, linf = T.calc_error_norms(u, semi, t=0.0, kind="convergence_test")
    # interpolation error of the degree-3 nodal representation, small but nonzero
    assert 0 < l2[0] < 1e-3 and 0 < linf[0] < 1e-2
    l2b, linfb = T.calc_error_norms(u, semi, u_ref=u)
    assert l2b[0] == 0.0 and linfb[0] == 0.0
    # host restatement of the same analysis
    from trixicuda.solver import lgl_basis_item
    import numpy.polynomial.legendre as npl  # noqa: F401

    N = semi.nnodes
    NA = 2 * (N - 1) + 1
    xa = lgl_basis_item(NA - 1, "nodes")
    wa = lgl_basis_item(NA - 1, "weights")
    x = semi.solver.basis.nodes
    V = np.array([[np.prod([(xa_i - x[m]) / (x[j] - x[m]) for m in range(N) if m != j]) for j in range(N)]
                  for xa_i in xa])
    uu = u.cpu().numpy().reshape(semi.nelements, N, N)
    coords = semi.containers.node_coordinates
    err2, errinf = 0.0, 0.0
    for e in range(semi.nelements):
        ua = V @ uu[e] @ V.T  # [ya, xa]
        x0, x1 = coords[e, 0, 0, 0], coords[e, 0, -1, 0]
        y0, y1 = coords[e, 0, 0, 1], coords[e, -1, 0, 1]
        X = x0 + 0.5 * (x1 - x0) * (xa + 1)
        Y = y0 + 0.5 * (y1 - y0) * (xa + 1)
        ex = 1 + 0.5 * np.sin(np.pi * (X[None, :] + Y[:, None]))
        J = (1.0 / semi.containers.inverse_jacobian[e]) ** 2
        err2 += np.sum((ex - ua) ** 2 * np.outer(wa, wa)) * J
        errinf = max(errinf, np.max(np.abs(ex - ua)))
    assert abs(l2[0] - np.sqrt(err2 / 4.0)) < 1e-12 * l2[0] + 1e-16
    assert abs(linf[0] - errinf) < 1e-12


def test_integrals_are_compensated(cuda):
    """The quadrature sums carry their rounding errors (TwoSum/TwoProduct):
    with +-1e16 on the two end nodes of every element (equal LGL weights up to
    their last bit) and O(1) values between, a plain FP64 sum loses the O(1)
    part entirely; the compensated sum matches the exact rational result."""
    from fractions import Fraction

    mesh = T.TreeMesh(-1.0, 1.0, initial_refinement_level=4)
    eq = T.LinearScalarAdvectionEquation1D(1.0)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_convergence_test, solver)
    E = semi.nelements
    u_host = np.ones((E, 4, 1))
    u_host[:, 0, 0] = 1.0e16
    u_host[:, 3, 0] = -1.0e16
    u = cuda.from_numpy(u_host).to(semi.device)
    got = T.integrate(u, semi, "state")[0]
    w = semi.solver.basis.weights
    J = 1.0 / semi.containers.inverse_jacobian
    exact = sum(Fraction(J[e]) * sum(Fraction(w[n]) * Fraction(u_host[e, n, 0]) for n in range(4)) for e in range(E))
    assert abs(Fraction(got) - exact) <= Fraction(1, 10 ** 14) * abs(exact), (got, float(exact))
    # a plain left-to-right FP64 sum per element is far off
    plain = sum(J[e] * sum(w[n] * u_host[e, n, 0] for n in range(4)) for e in range(E))
    assert abs(plain - float(exact)) > 1e-3 * abs(float(exact))
