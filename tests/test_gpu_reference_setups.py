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
