"""flux_shima_etal, flux_hll and flux_hlle in the CPU oracle (no GPU), as the reference's
tests use them: flux_shima_etal as the DG volume flux of shock capturing
(test/tree_dgsem_{1,2}d/euler_shock.jl), flux_hll as the surface flux of the
weak form (test/tree_dgsem_3d/euler_convergence.jl).  Pins: free-stream
preservation (consistency, also across mortars), discrete conservation on
periodic meshes, and the convergence order of the manufactured solution."""
import ctypes as C

import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import Oracle, basis
from problems import host_problem


def _const_state(s, orc):
    eq = s.equations
    d = eq.ndims
    state = eq.prim2cons(np.array([1.2]), np.array([[0.3], [-0.2], [0.1]][:d]), np.array([0.9]))[:, 0]
    nn = (s.solver.polydeg + 1) ** d
    return np.broadcast_to(state, (s.containers.nelements, nn, eq.nvariables)).copy()


CASES = [
    ("euler_sc", 1, 4, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_sc", 2, 3, True, dict(volume_flux=T.flux_shima_etal)),
    ("euler_sc", 3, 2, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_fd", 2, 2, True, dict(volume_flux=T.flux_shima_etal, surface_flux=T.flux_hll)),
    ("euler_weak", 3, 1, True, dict(surface_flux=T.flux_hll)),
    ("euler_fd", 3, 1, False, dict(surface_flux=T.flux_hll)),
    ("adv_weak", 2, 2, True, dict(surface_flux=T.flux_hll)),
    ("euler_weak", 2, 2, True, dict(surface_flux=T.flux_hlle)),
    ("euler_sc", 3, 1, True, dict(fv_flux=T.flux_hlle, surface_flux=T.flux_hlle)),
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}d-{'-'.join(f.name for f in c[4].values())}" for c in CASES])
def test_free_stream(case):
    kind, d, level, refined, kw = case
    s, orc, u = host_problem(kind, d, level, refined=refined, **kw)
    if kind.startswith("adv"):
        u = np.ones_like(u)
    else:
        u = _const_state(s, orc).reshape(u.shape)
    du = orc.rhs(u, 0.0)
    assert np.max(np.abs(du)) < 1e-12


CONS = CASES[1:5] + CASES[7:]


@pytest.mark.parametrize("case", CONS, ids=[f"{c[0]}-{c[1]}d-{'-'.join(f.name for f in c[4].values())}" for c in CONS])
def test_conservation(case):
    """sum_e J_e sum_i w_i du_i = 0 per conserved variable on periodic meshes
    (also across mortars: the L2 mortar projection of the surface flux is
    conservative)."""
    kind, d, level, refined, kw = case
    s, orc, u = host_problem(kind, d, level, refined=refined, **kw)
    u = u * (1.0 + 0.01 * np.random.default_rng(3).standard_normal(u.shape))
    du = orc.rhs(u, 0.0)
    w1 = basis(s.solver.polydeg)["weights"]
    wn = w1
    for _ in range(d - 1):
        wn = np.multiply.outer(wn, w1)
    wn = np.ascontiguousarray(wn.T).reshape(-1)
    J = (1.0 / s.containers.inverse_jacobian) ** d
    nv = s.equations.nvariables
    tot = np.einsum("e,n,env->v", J, wn, du.reshape(len(J), -1, nv))
    scale = np.einsum("e,n,env->v", J, wn, np.abs(du.reshape(len(J), -1, nv)))
    assert np.all(np.abs(tot) <= 1e-13 * np.maximum(scale, 1e-300)), (tot, scale)


def _eoc_error(level, surface_flux, d=2, p=3, t_end=0.1):
    """Periodic manufactured solution of the Euler equations (rho = rho v_d =
    2 + 0.1 sin(pi (sum x - t)), E = rho^2 on [0, 2]^d) with its source term."""
    mesh = T.TreeMesh((0.0,) * d, (2.0,) * d, initial_refinement_level=level)
    eq = {2: T.CompressibleEulerEquations2D, 3: T.CompressibleEulerEquations3D}[d](1.4)
    solver = T.DGSEMGPU(polydeg=p, surface_flux=surface_flux)
    cont = mesh.build_containers(solver.basis.nodes)
    orc = Oracle(cont, d, p, eq.nvariables, eq.code, gamma=1.4, volume_integral=0, surface_flux=surface_flux.code,
                 source_terms=1)
    x = cont.node_coordinates.reshape(-1, d).T
    shape = (cont.nelements,) + (p + 1,) * d + (eq.nvariables,)
    u = np.ascontiguousarray(T.initial_condition_convergence_test(x, 0.0, eq).T.reshape(shape))
    k = np.zeros_like(u)
    h = 2.0 / 2 ** level
    nsteps = int(np.ceil(t_end / (0.4 * h / (p + 1) / 3.0)))
    pd = C.POINTER(C.c_double)
    orc.lib.oracle_rk_ck2n54(orc._h, u.ctypes.data_as(pd), k.ctypes.data_as(pd), 0.0, t_end / nsteps, nsteps)
    ue = T.initial_condition_convergence_test(x, t_end, eq).T.reshape(shape)
    return float(np.sqrt(np.mean((u - ue) ** 2)))


@pytest.mark.parametrize("flux", [T.flux_hll, T.flux_hlle], ids=lambda f: f.name)
def test_hll_convergence_order(flux):
    """Weak form with flux_hll / flux_hlle converges at about polydeg + 1."""
    e0, e1 = _eoc_error(2, flux), _eoc_error(3, flux)
    assert np.log2(e0 / e1) > 3.3, (e0, e1)
