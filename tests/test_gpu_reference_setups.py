"""More of the reference's Euler test set-ups on the GPU against the CPU
oracle (FP64, 1e-12 relative; RK steps 1e-11 on the increment):
* test/tree_dgsem_1d/euler_blast_wave.jl -- the strong blast wave (its
  initial condition is defined in that test: p = 1e-3 outside r = 0.5),
  shock capturing on density_pressure, level 6;
* test/tree_dgsem_{1,2}d/euler_source_terms.jl -- the weak form with
  flux_lax_friedrichs and source_terms_convergence_test on a periodic mesh;
* test/tree_dgsem_3d/euler_mortar.jl -- the same on a refined 3D mesh, so
  source terms and mortars meet in one kernel."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def initial_condition_blast_wave(x, t, eq):
    """Strong blast wave at the origin: inside |x| <= 0.5 rho 1.1691, velocity
    0.1882 away from the origin, p 1.245; outside rho 1, v 0, p 1e-3."""
    x1 = x[0]
    inside = np.abs(x1) <= 0.5
    cos_phi = np.where(x1 > 0, 1.0, -1.0)
    rho = np.where(inside, 1.1691, 1.0)
    v1 = np.where(inside, 0.1882 * cos_phi, 0.0)
    p = np.where(inside, 1.245, 1.0e-3)
    return eq.prim2cons(rho, v1[None, :], p)


def _check(semi, orc, cuda, steps=2, dt=1e-3):
    u_host = semi.compute_coefficients_host()
    u = cuda.from_numpy(u_host).to(semi.device)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), 1e-12, "rhs")
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.0, dt, steps, semi)
    T.synchronize(semi)
    uo, _ = orc.rk_ck2n54(u_host, 0.0, dt, steps)
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, 1e-11, "rk increment")


def test_euler_blast_wave_1d(cuda):
    eq = T.CompressibleEulerEquations1D(1.4)
    ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs, volume_integral=vi)
    mesh = T.TreeMesh((-2.0,), (2.0,), initial_refinement_level=6)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, initial_condition_blast_wave, solver)
    orc = Oracle.from_semi(semi)
    # the jumps at |x| = 0.5 lie on element interfaces at level 6: every element
    # starts constant and the indicator is zero; after a few steps it fires
    u0 = semi.compute_coefficients_host()
    assert np.count_nonzero(orc.indicator(u0)) == 0
    u20, _ = orc.rk_ck2n54(u0, 0.0, 1e-3, 20)
    alpha = cuda.zeros(semi.nelements, dtype=cuda.float64, device=semi.device)
    T.cuda_indicator(cuda.from_numpy(u20).to(semi.device), alpha, semi)
    a_o = orc.indicator(u20)
    assert np.count_nonzero(a_o) > 0
    assert np.max(np.abs(alpha.cpu().numpy() - a_o)) < 1e-12
    _check(semi, orc, cuda, dt=1e-4)


@pytest.mark.parametrize("d,level,polydeg,refined", [(1, 4, 4, False), (2, 4, 3, False), (3, 2, 3, True)])
def test_euler_source_terms_periodic(d, level, polydeg, refined, cuda):
    eq = {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
          3: T.CompressibleEulerEquations3D}[d](1.4)
    patches = [dict(type="box", coordinates_min=(0.5,) * d, coordinates_max=(1.5,) * d)] if refined else []
    mesh = T.TreeMesh((0.0,) * d, (2.0,) * d, initial_refinement_level=level, refinement_patches=patches)
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=T.flux_lax_friedrichs)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_convergence_test, solver,
                                             source_terms=T.source_terms_convergence_test)
    orc = Oracle.from_semi(semi)
    if refined:
        assert semi.containers.nmortars > 0
    _check(semi, orc, cuda)


@pytest.mark.parametrize("d,level,precision", [(3, 2, "fp64"), (2, 3, "fp64"), (3, 2, "mixed")])
def test_euler_convergence_euler_gravity(d, level, precision, cuda):
    """test/tree_dgsem_3d/euler_convergence.jl: gamma = 2,
    initial_condition_eoc_test_coupled_euler_gravity,
    source_terms_eoc_test_euler, flux_hll surface flux, weak form, periodic
    [0, 2]^3 at level 2 (and the 2D analogue): rhs, the stage functions and RK
    steps against the oracle; FP32-mixed within the mixed bar (5e-4)."""
    eq = {2: T.CompressibleEulerEquations2D, 3: T.CompressibleEulerEquations3D}[d](2.0)
    mesh = T.TreeMesh((0.0,) * d, (2.0,) * d, initial_refinement_level=level)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_hll, volume_integral=T.VolumeIntegralWeakForm())
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_eoc_test_coupled_euler_gravity, solver,
                                             source_terms=T.source_terms_eoc_test_euler, precision=precision)
    orc = Oracle.from_semi(semi)
    if precision == "mixed":
        u_host = semi.compute_coefficients_host()
        u = cuda.from_numpy(u_host).to(semi.device)
        du = cuda.empty_like(u)
        T.rhs_gpu(du, u, semi, 0.0)
        T.synchronize(semi)
        assert_rel(du.cpu().numpy(), orc.rhs(u_host), 5e-4, "mixed rhs")
        return
    _check(semi, orc, cuda)
    # stage by stage, as the reference test does
    u_host = semi.compute_coefficients_host()
    u = cuda.from_numpy(u_host).to(semi.device)
    du = cuda.empty_like(u)
    T.cuda_volume_integral(du, u, semi)
    du_o = orc.volume_integral(u_host)
    assert_rel(du.cpu().numpy(), du_o, 1e-12, "volume integral")
    T.cuda_prolong2interfaces(u, semi)
    T.cuda_interface_flux(semi)
    T.cuda_prolong2boundaries(u, semi)
    T.cuda_boundary_flux(0.0, semi)
    T.cuda_prolong2mortars(u, semi)
    T.cuda_mortar_flux(semi)
    sfv_o = orc.interface_flux(orc.prolong2interfaces(u_host))
    sfv = semi.container(T._lib.CONTAINER_SURFACE_FLUX_VALUES)
    assert_rel(sfv.cpu().numpy(), sfv_o, 1e-12, "surface_flux_values (flux_hll)")
    T.cuda_surface_integral(du, semi)
    T.cuda_jacobian(du, semi)
    T.cuda_sources(du, u, 0.0, semi)
    T.synchronize(semi)
    du_o = orc.sources(orc.jacobian(orc.surface_integral(du_o, sfv_o)), 0.0)
    assert_rel(du.cpu().numpy(), du_o, 1e-12, "after cuda_sources")
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), 1e-12, "staged == oracle rhs")
