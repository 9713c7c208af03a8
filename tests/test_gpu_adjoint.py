"""Discrete adjoint: the VJP of the rhs is the transpose of its Jacobian
(dot-product test against finite-difference JVPs), and the gradient of an RK
solve matches central finite differences along seeded random directions,
with and without checkpoint recomputation."""
import numpy as np
import pytest

import trixicuda as T
from trixicuda import adjoint as ADJ
from problems import make

pytestmark = pytest.mark.gpu


def _semi(kind, d, level, p=3, ic=None, **kw):
    mesh, eq, ic0, solver, _ = make(kind, d, level, polydeg=p, **kw)
    return T.SemidiscretizationHyperbolicGPU(mesh, eq, ic or ic0, solver)


CASES = [("euler_fd", 2, 2, 3, None, {}), ("euler_fd", 3, 1, 3, None, {}), ("euler_fd", 2, 2, 4, None, {}),
         ("euler_fd", 2, 2, 3, "blast", {}),  # large ratios: the log branch of the means
         ("euler_fd", 2, 2, 3, None, dict(surface_flux=T.flux_central, volume_flux=T.flux_central)),
         # one flux with primitive-variable cotangents, the other with conservative ones
         ("euler_fd", 2, 2, 3, None, dict(surface_flux=T.flux_ranocha, volume_flux=T.flux_central)),
         ("euler_fd", 2, 2, 4, None, dict(surface_flux=T.flux_central, volume_flux=T.flux_ranocha)),
         ("adv_weak", 2, 2, 3, None, {}), ("adv_weak", 1, 3, 3, None, {}), ("adv_fd", 3, 1, 3, None, {}),
         ("adv_weak", 2, 2, 3, None, dict(surface_flux=T.flux_central)),
         # flux_hll on linear advection is the upwind flux (signal speeds lmin = lmax = a)
         ("adv_weak", 2, 2, 3, None, dict(surface_flux=T.flux_hll)),
         ("adv_weak", 1, 3, 3, None, dict(surface_flux=T.flux_hll))]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}d-p{c[3]}-{c[4]}-{len(c[5])}" for c in CASES])
def test_rhs_vjp_is_jacobian_transpose(case, cuda):
    kind, d, level, p, icname, kw = case
    semi = _semi(kind, d, level, p, T.initial_condition_weak_blast_wave if icname else None, **kw)
    u = semi.compute_coefficients()
    rng = np.random.default_rng(3)
    for trial in range(3):
        v = cuda.from_numpy(rng.standard_normal(u.shape)).to(u.device)
        lam = cuda.from_numpy(rng.standard_normal(u.shape)).to(u.device)
        h = 1e-6 * float(u.abs().max()) / float(v.abs().max())
        fp, fm = cuda.empty_like(u), cuda.empty_like(u)
        T.rhs_gpu(fp, u + h * v, semi, 0.0)
        T.rhs_gpu(fm, u - h * v, semi, 0.0)
        jv = (fp - fm) / (2 * h)
        ubar = cuda.empty_like(u)
        ADJ.rhs_vjp(ubar, u, lam, semi)
        T.synchronize(semi)
        lhs = float((lam * jv).sum())
        rhs = float((ubar * v).sum())
        scale = float((lam.abs() * jv.abs()).sum())
        assert abs(lhs - rhs) <= 1e-6 * scale, (trial, lhs, rhs)


def _rho_target(semi, cuda):
    x = semi.containers.node_coordinates.reshape(-1, semi.mesh.ndims).T
    f = T.equations.FourierField(semi.mesh.ndims, 4, 77, -2.0, 2.0)
    return cuda.from_numpy(1.0 + 0.05 * f(x)).to(semi.device)


@pytest.mark.parametrize("snapshots", [0, 3, 100])
def test_solve_gradient_matches_finite_differences(snapshots, cuda):
    semi = _semi("euler_fd", 2, 3, 3)
    u0 = semi.compute_coefficients()
    rt = _rho_target(semi, cuda)
    dt = 0.3 * T.max_dt(u0, semi)
    nsteps = 12
    J, grad, nrec = ADJ.gradient_density_l2(semi, u0, rt, dt, nsteps, snapshots)
    if snapshots >= nsteps - 1:
        assert nrec == 0
    rng = np.random.default_rng(11)
    for _ in range(4):
        dirn = cuda.from_numpy(rng.standard_normal(u0.shape)).to(u0.device)
        h = 1e-6
        vals = []
        for sgn in (1, -1):
            u = (u0 + sgn * h * dirn).contiguous()
            k = cuda.zeros_like(u)
            T.rk_steps(u, k, 0.0, dt, nsteps, semi)
            vals.append(ADJ.objective_density_l2(u, rt, semi, grad=False)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = float((grad * dirn).sum())
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-12), (fd, ad)


def test_checkpointing_is_exact(cuda):
    semi = _semi("euler_fd", 2, 2, 3)
    u0 = semi.compute_coefficients()
    rt = _rho_target(semi, cuda)
    dt = 0.3 * T.max_dt(u0, semi)
    grads = [ADJ.gradient_density_l2(semi, u0, rt, dt, 20, s)[1] for s in (0, 2, 5, 19)]
    for g in grads[1:]:
        assert cuda.equal(g, grads[0])


def test_autograd_function(cuda):
    semi = _semi("euler_fd", 2, 2, 3)
    u0 = semi.compute_coefficients().requires_grad_(True)
    rt = _rho_target(semi, cuda)
    dt = 0.3 * T.max_dt(u0.detach(), semi)
    uT = ADJ.rk_solve_autograd(u0, semi, dt, 6, 2)
    J, g = ADJ.objective_density_l2(uT.detach(), rt, semi)
    uT.backward(g)
    _, g_ref, _ = ADJ.gradient_density_l2(semi, u0.detach(), rt, dt, 6, 2)
    assert cuda.allclose(u0.grad, g_ref, rtol=0, atol=0)


def test_full_size_c4_gradient_matches_fd(cuda):
    """The adjoint configuration at full size: 2D Euler level 6, polydeg 4,
    flux_ranocha, J = 1/2 int (rho(T) - rho_target)^2 after 200 CK2N54 steps,
    binomial checkpointing with 15 snapshots; the gradient must match central
    finite differences (h = 1e-6) to 1e-6 along 16 seeded random directions."""
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEMGPU(polydeg=4, surface_flux=T.flux_ranocha,
                        volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=6)
    ic = T.initial_condition_fourier_euler(eq, seed=20261203, kmax=8)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver)
    u0 = semi.compute_coefficients()
    x = semi.containers.node_coordinates.reshape(-1, 2).T
    rt = cuda.from_numpy(1.0 + 0.05 * T.equations.FourierField(2, 4, 4242, -2.0, 2.0)(x)).to(u0.device)
    dt = 0.5 * T.max_dt(u0, semi)
    nsteps = 200
    J, grad, nrec = ADJ.gradient_density_l2(semi, u0, rt, dt, nsteps, 15)
    assert nrec > 0
    rng = np.random.default_rng(20261203)
    for _ in range(16):
        dirn = cuda.from_numpy(rng.standard_normal(u0.shape)).to(u0.device)
        vals = []
        for sgn in (1, -1):
            u = (u0 + sgn * 1e-6 * dirn).contiguous()
            k = cuda.zeros_like(u)
            T.rk_steps(u, k, 0.0, dt, nsteps, semi)
            vals.append(ADJ.objective_density_l2(u, rt, semi, grad=False)[0])
        fd = (vals[0] - vals[1]) / 2e-6
        ad = float((grad * dirn).sum())
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
