"""The set-up of the reference's test/tree_dgsem_2d/euler_blob_mortar.jl on
the GPU against the CPU oracle: a dense blob in a Mach 2.7 stream (gamma =
5/3), shock capturing with the Hennemann-Gassner indicator on `pressure`
(alpha_max 0.05, alpha_min 1e-4, smoothing), flux_ranocha volume flux,
flux_lax_friedrichs surface and FV fluxes, a TreeMesh [-32, 32]^2 of level 4
refined twice in the box [-40, 40] x [-5, 5] (mortars between levels 4-5-6)."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def initial_condition_blob(x, t, eq):
    """The blob of the reference test (density contrast 10, radius 1, centre
    (-15, 0), smoothed by tanh profiles of slope 2; background Mach 2.7)."""
    R, dens0, chi = 1.0, 1.0, 10.0
    tau_cr = 1.0 / 1.6
    velx0 = 2 * R * np.sqrt(chi) / tau_cr
    c = velx0 / 2.7
    p0 = c * c * dens0 / eq.gamma
    r = np.sqrt((x[0] + 15.0) ** 2 + x[1] ** 2)
    blob = 0.5 * (1 + (np.tanh(2 * (r + R)) - (np.tanh(2 * (r - R)) + 1)))
    dens = dens0 + (chi - 1) * blob
    velx = velx0 - velx0 * blob
    return eq.prim2cons(dens, np.stack([velx, np.zeros_like(velx)]), np.full_like(dens, p0))


def _semi(precision="fp64"):
    eq = T.CompressibleEulerEquations2D(5.0 / 3.0)
    ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.05, alpha_min=0.0001, alpha_smooth=True,
                                      variable=T.pressure)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs, volume_integral=vi)
    box = dict(type="box", coordinates_min=(-40.0, -5.0), coordinates_max=(40.0, 5.0))
    mesh = T.TreeMesh((-32.0, -32.0), (32.0, 32.0), initial_refinement_level=4, refinement_patches=[box, box])
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, initial_condition_blob, solver, precision=precision)
    return semi, Oracle.from_semi(semi)


def test_blob_indicator_on_pressure(cuda):
    semi, orc = _semi()
    u_host = semi.compute_coefficients_host()
    u = cuda.from_numpy(u_host).to(semi.device)
    alpha = cuda.zeros(semi.nelements, dtype=cuda.float64, device=semi.device)
    T.cuda_indicator(u, alpha, semi)
    a_o = orc.indicator(u_host)
    assert np.max(np.abs(alpha.cpu().numpy() - a_o)) < 1e-12
    assert np.count_nonzero(a_o) > 0  # the blob's edge triggers the indicator


@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-12), ("mixed", 5e-4)])
def test_blob_rhs_and_rk(precision, rtol, cuda):
    semi, orc = _semi(precision)
    u_host = semi.compute_coefficients_host()
    u = cuda.from_numpy(u_host).to(semi.device)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), rtol, "rhs")
    k = cuda.zeros_like(u)
    dt = 1e-3
    T.rk_steps(u, k, 0.0, dt, 2, semi)
    T.synchronize(semi)
    uo, _ = orc.rk_ck2n54(u_host, 0.0, dt, 2)
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, rtol * 10, "rk increment")
