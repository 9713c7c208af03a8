"""flux_shima_etal (volume flux), flux_hll and flux_hlle (surface fluxes) on the GPU
against the CPU oracle.  Set-ups follow the reference's
test/tree_dgsem_{1,2}d/euler_shock.jl (shock capturing with flux_shima_etal
as the DG volume flux, flux_lax_friedrichs surface and FV fluxes) and
test/tree_dgsem_3d/euler_convergence.jl (weak form, flux_hll, with a source
term), plus flux differencing, mortars, FP32-mixed and ideal GLM-MHD with
flux_hll.  FP64 to 1e-12, mixed to 5e-4 (2-norm), as the other parity tests."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from oracle.oracle import Oracle
from problems import semi_and_oracle

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12
RTOL_MIXED = 5e-4

CASES = [
    ("euler_sc", 1, 5, 3, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_sc", 2, 4, 3, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_sc", 2, 3, 3, True, dict(volume_flux=T.flux_shima_etal)),
    ("euler_sc", 3, 2, 3, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_fd", 2, 3, 3, True, dict(volume_flux=T.flux_shima_etal, surface_flux=T.flux_hll)),
    ("euler_fd", 3, 2, 4, False, dict(volume_flux=T.flux_shima_etal)),
    ("euler_weak", 3, 2, 3, False, dict(surface_flux=T.flux_hll)),
    ("euler_weak", 2, 3, 3, True, dict(surface_flux=T.flux_hll)),
    ("euler_sc", 2, 3, 3, False, dict(fv_flux=T.flux_hll, surface_flux=T.flux_hll)),
    ("adv_weak", 2, 3, 3, True, dict(surface_flux=T.flux_hll)),
    ("euler_weak", 2, 3, 3, True, dict(surface_flux=T.flux_hlle)),
    ("euler_sc", 3, 2, 3, False, dict(fv_flux=T.flux_hlle, surface_flux=T.flux_hlle)),
    ("euler_fd", 1, 4, 3, False, dict(surface_flux=T.flux_hlle)),
    ("euler_fd", 3, 1, 4, True, dict(surface_flux=T.flux_hlle)),
]


def _ids(c):
    return f"{c[0]}-{c[1]}d-L{c[2]}-p{c[3]}{'-ref' if c[4] else ''}-" + "-".join(f.name for f in c[5].values())


def _u0(semi, cuda, perturb=False):
    u = semi.compute_coefficients_host()
    if perturb:
        u = np.ascontiguousarray(u * (1.0 + 0.01 * np.random.default_rng(9).standard_normal(u.shape)))
    return u, cuda.from_numpy(u).to(semi.device)


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_rhs_matches_oracle(case, cuda):
    kind, d, level, p, refined, kw = case
    semi, orc = semi_and_oracle(kind, d, level, polydeg=p, refined=refined, **kw)
    u_host, u = _u0(semi, cuda, perturb=True)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL64, "rhs")


MIXED = [CASES[1], CASES[4], CASES[6], CASES[10], CASES[11]]


@pytest.mark.parametrize("case", MIXED, ids=[_ids(c) for c in MIXED])
def test_mixed_rhs_close_to_oracle(case, cuda):
    kind, d, level, p, refined, kw = case
    semi, orc = semi_and_oracle(kind, d, level, polydeg=p, refined=refined, precision="mixed", **kw)
    u_host, u = _u0(semi, cuda, perturb=True)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL_MIXED, "mixed rhs")


def test_hll_weak_form_with_source_terms(cuda):
    """The euler_convergence.jl shape: weak form, flux_hll, periodic, a
    manufactured source term (here the convergence-test source of this
    library), RK steps against the oracle."""
    mesh = T.TreeMesh((0.0,) * 3, (2.0,) * 3, initial_refinement_level=2)
    eq = T.CompressibleEulerEquations3D(1.4)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_hll)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_convergence_test, solver,
                                             source_terms=T.source_terms_convergence_test)
    orc = Oracle.from_semi(semi)
    u_host, u = _u0(semi, cuda)
    k = cuda.zeros_like(u)
    dt = 2e-3
    T.rk_steps(u, k, 0.0, dt, 3, semi)
    T.synchronize(semi)
    uo, _ = orc.rk_ck2n54(u_host, 0.0, dt, 3)
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, 1e-11, "rk increment")


def test_shima_rejected_as_surface_flux(cuda):
    mesh, eq = T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=2), T.CompressibleEulerEquations2D(1.4)
    with pytest.raises(T.TrixiError):
        T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_weak_blast_wave,
                                          T.DGSEMGPU(polydeg=3, surface_flux=T.flux_shima_etal))


MHD_MORTAR = [(T.flux_hll, 2, "fp64"), (T.flux_hlle, 2, "fp64"), (T.flux_hlle, 3, "fp64"), (T.flux_hlle, 2, "mixed"),
              (T.flux_hlle, 1, "fp64")]


@pytest.mark.parametrize("flux,d,precision", MHD_MORTAR, ids=[f"{f.name}-{d}d-{p}" for f, d, p in MHD_MORTAR])
def test_mhd_alfven_wave_mortar(flux, d, precision, cuda):
    """test/tree_dgsem_{2,3}d/mhd_alfven_wave_mortar.jl: flux_hlle (Einfeldt
    speeds with the Cargo-Gallice average) or flux_hll (naive fast
    magnetosonic estimates) as the surface flux paired with the Powell term,
    flux_hindenlang_gassner volume flux, a refined box; the fused rhs and the
    stage-by-stage API."""
    lo, hi = {1: (0.0, 1.0), 2: (0.0, np.sqrt(2.0)), 3: (-1.0, 1.0)}[d]
    level = {1: 4, 2: 3, 3: 2}[d]
    patches = [dict(type="box", coordinates_min=(lo + 0.25 * (hi - lo),) * d,
                    coordinates_max=(lo + 0.75 * (hi - lo),) * d)] if d > 1 else []
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches)
    eq = {1: T.IdealGlmMhdEquations1D, 2: T.IdealGlmMhdEquations2D, 3: T.IdealGlmMhdEquations3D}[d](5.0 / 3.0, 0.7)
    pair = (lambda f: (f, T.flux_nonconservative_powell)) if d > 1 else (lambda f: f)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=pair(flux),
                        volume_integral=T.VolumeIntegralFluxDifferencing(pair(T.flux_hindenlang_gassner)))
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_convergence_test, solver,
                                             precision=precision)
    assert d == 1 or semi.containers.nmortars > 0
    orc = Oracle.from_semi(semi)
    u_host, u = _u0(semi, cuda, perturb=True)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    rtol = RTOL64 if precision == "fp64" else RTOL_MIXED
    ref = orc.rhs(u_host)
    assert_rel(du.cpu().numpy(), ref, rtol, f"mhd {flux.name} rhs")
    if precision == "fp64":
        du2 = cuda.empty_like(u)
        T.cuda_volume_integral(du2, u, semi)
        T.cuda_prolong2interfaces(u, semi)
        T.cuda_interface_flux(semi)
        T.cuda_prolong2mortars(u, semi)
        T.cuda_mortar_flux(semi)
        T.cuda_surface_integral(du2, semi)
        T.cuda_jacobian(du2, semi)
        T.synchronize(semi)
        assert_rel(du2.cpu().numpy(), ref, RTOL64, f"staged mhd {flux.name} rhs")


def test_hlle_rejections(cuda):
    """flux_hlle is defined for Euler and MHD, as a surface or FV flux."""
    mesh = T.TreeMesh((0.0, 0.0), (2.0, 2.0), initial_refinement_level=2)
    adv = T.LinearScalarAdvectionEquation2D((1.0, 0.5))
    with pytest.raises(T.TrixiError):
        T.SemidiscretizationHyperbolicGPU(mesh, adv, T.initial_condition_convergence_test,
                                          T.DGSEMGPU(polydeg=3, surface_flux=T.flux_hlle))
    eq = T.CompressibleEulerEquations2D(1.4)
    with pytest.raises(T.TrixiError):
        T.SemidiscretizationHyperbolicGPU(mesh, eq, T.initial_condition_weak_blast_wave, T.DGSEMGPU(
            polydeg=3, volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_hlle)))
