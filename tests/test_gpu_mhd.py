"""Ideal GLM-MHD on the GPU (through the C ABI) against the CPU oracle.
Mirrors the reference's MHD tests: test/tree_dgsem_{1,2,3}d/mhd_ec.jl
(flux_hindenlang_gassner volume and surface), mhd_alfven_wave.jl
(flux_central or flux_hindenlang_gassner volume, flux_lax_friedrichs surface),
mhd_alfven_wave_mortar.jl (refined box, mortars) and mhd_shock.jl (shock
capturing, polydeg 4), each flux paired with flux_nonconservative_powell in
2D/3D.  FP64 to 1e-12 relative (2-norm), FP32-mixed to 5e-4, as the other
parity tests."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12
RTOL_MIXED = 5e-4
EQS = {1: T.IdealGlmMhdEquations1D, 2: T.IdealGlmMhdEquations2D, 3: T.IdealGlmMhdEquations3D}


def _pair(f, d):
    return (f, T.flux_nonconservative_powell) if d > 1 else f


def _semi(setup, d, level, polydeg=3, refined=False, precision="fp64", c_h=0.8):
    if setup == "alfven":
        gamma, ic = 5.0 / 3.0, T.initial_condition_convergence_test
        lo, hi = {1: (0.0, 1.0), 2: (0.0, np.sqrt(2.0)), 3: (-1.0, 1.0)}[d]
    else:
        gamma, ic = 1.4, T.initial_condition_weak_blast_wave
        lo, hi = (0.0, 1.0) if d == 1 else (-2.0, 2.0)
    patches = [dict(type="box", coordinates_min=(lo + 0.25 * (hi - lo),) * d,
                    coordinates_max=(lo + 0.75 * (hi - lo),) * d)] if refined else []
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches)
    eq = EQS[d](gamma, c_h)
    if setup == "ec":            # mhd_ec.jl
        sflux, vi = _pair(T.flux_hindenlang_gassner, d), T.VolumeIntegralFluxDifferencing(
            _pair(T.flux_hindenlang_gassner, d))
    elif setup == "alfven":      # mhd_alfven_wave.jl (2D: flux_central volume flux)
        vf = T.flux_central if d == 2 else T.flux_hindenlang_gassner
        sflux, vi = _pair(T.flux_lax_friedrichs, d), T.VolumeIntegralFluxDifferencing(_pair(vf, d))
    else:                        # mhd_shock.jl
        ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
        sflux = _pair(T.flux_hindenlang_gassner, d)
        vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=_pair(T.flux_hindenlang_gassner, d),
                                              volume_flux_fv=sflux)
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=sflux, volume_integral=vi)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    return semi, Oracle.from_semi(semi)


def _u(semi, cuda, perturb=True):
    u = semi.compute_coefficients_host()
    if perturb:  # traces jump across interfaces
        u = np.ascontiguousarray(u * (1.0 + 0.01 * np.random.default_rng(5).standard_normal(u.shape)))
    return u, cuda.from_numpy(u).to(semi.device)


CASES = [
    ("ec", 1, 4, 3, False),
    ("alfven", 1, 2, 4, False),
    ("ec", 2, 3, 3, False),
    ("alfven", 2, 3, 3, False),
    ("alfven", 2, 3, 3, True),
    ("shock", 2, 3, 4, False),
    ("shock", 2, 2, 4, True),
    ("ec", 3, 2, 3, False),
    ("alfven", 3, 2, 3, False),
    ("alfven", 3, 1, 3, True),
    ("shock", 3, 2, 4, False),
] + [("ec", 2, 2, p, True) for p in (1, 2, 4)] + [("ec", 3, 1, p, False) for p in (1, 2)]


def _ids(c):
    return f"{c[0]}-{c[1]}d-L{c[2]}-p{c[3]}{'-ref' if c[4] else ''}"


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_mhd_rhs_matches_oracle(case, cuda):
    setup, d, level, p, refined = case
    semi, orc = _semi(setup, d, level, p, refined)
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL64, "mhd rhs")


MIXED = [("alfven", 2, 3, 3, True), ("ec", 3, 2, 3, False), ("shock", 2, 3, 4, False), ("ec", 1, 4, 3, False)]


@pytest.mark.parametrize("case", MIXED, ids=[_ids(c) for c in MIXED])
def test_mhd_mixed_rhs_close_to_oracle(case, cuda):
    setup, d, level, p, refined = case
    semi, orc = _semi(setup, d, level, p, refined, precision="mixed")
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL_MIXED, "mixed mhd rhs")


STAGE_CASES = [("alfven", 2, 3, 3, True), ("shock", 2, 3, 4, False), ("alfven", 3, 1, 3, True), ("ec", 1, 3, 3, False)]


@pytest.mark.parametrize("case", STAGE_CASES, ids=[_ids(c) for c in STAGE_CASES])
def test_mhd_stages_match_oracle(case, cuda):
    """cuda_volume_integral! (with the nonconservative volume terms),
    cuda_interface_flux! (each side its own 0.5 Phi), cuda_mortar_flux!
    (primary / secondary), surface integral and Jacobian, stage by stage as
    the reference's MHD tests call them."""
    setup, d, level, p, refined = case
    semi, orc = _semi(setup, d, level, p, refined)
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    alpha = orc.indicator(u_host) if setup == "shock" else None
    T.cuda_volume_integral(du, u, semi)
    du_o = orc.volume_integral(u_host, alpha)
    assert_rel(du.cpu().numpy(), du_o, RTOL64, "volume integral")
    T.cuda_prolong2interfaces(u, semi)
    iu_o = orc.prolong2interfaces(u_host)
    assert_rel(semi.container(T._lib.CONTAINER_INTERFACES_U).cpu().numpy(), iu_o, 0.0, "interfaces.u")
    T.cuda_interface_flux(semi)
    sfv_o = orc.interface_flux(iu_o)
    T.cuda_prolong2mortars(u, semi)
    if semi.containers.nmortars:
        orc.mortar_flux(orc.prolong2mortars(u_host), sfv_o)
    T.cuda_mortar_flux(semi)
    assert_rel(semi.container(T._lib.CONTAINER_SURFACE_FLUX_VALUES).cpu().numpy(), sfv_o, RTOL64,
               "surface_flux_values")
    T.cuda_surface_integral(du, semi)
    du_o = orc.surface_integral(du_o, sfv_o)
    T.cuda_jacobian(du, semi)
    du_o = orc.jacobian(du_o)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), du_o, RTOL64, "staged rhs")
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL64, "staged == oracle rhs")


def test_mhd_indicator_matches_oracle(cuda):
    semi, orc = _semi("shock", 2, 4, 4, False)
    u_host, u = _u(semi, cuda, perturb=False)
    alpha = cuda.zeros(semi.nelements, dtype=cuda.float64, device=semi.device)
    T.cuda_indicator(u, alpha, semi)
    a_o = orc.indicator(u_host)
    assert np.max(np.abs(alpha.cpu().numpy() - a_o)) < 1e-12
    assert np.count_nonzero(a_o) > 0


@pytest.mark.parametrize("case,precision,rtol", [(("alfven", 2, 3, 3, True), "fp64", RTOL64),
                                                 (("shock", 3, 2, 4, False), "fp64", RTOL64),
                                                 (("alfven", 2, 3, 3, False), "mixed", RTOL_MIXED)])
def test_mhd_rk_steps_match_oracle(case, precision, rtol, cuda):
    setup, d, level, p, refined = case
    semi, orc = _semi(setup, d, level, p, refined, precision=precision)
    u_host, u = _u(semi, cuda, perturb=False)
    k = cuda.zeros_like(u)
    dt = 0.1 / float(np.max(semi.containers.inverse_jacobian)) / (p + 1) / 2.0
    T.rk_steps(u, k, 0.0, dt, 3, semi)
    T.synchronize(semi)
    uo, _ = orc.rk_ck2n54(u_host, 0.0, dt, 3)
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, rtol * 10, "rk increment")


def test_mhd_glm_speed_update(cuda):
    """trixi_set_glm_speed between calls (a GlmSpeedCallback): the rhs follows
    the new c_h."""
    semi, _ = _semi("ec", 2, 3, 3, False, c_h=0.8)
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.set_glm_speed(semi, 1.7)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    orc = Oracle.from_semi(semi)  # reads equations.c_h = 1.7
    assert semi.equations.c_h == 1.7
    assert_rel(du.cpu().numpy(), orc.rhs(u_host), RTOL64, "rhs after set_glm_speed")


def test_mhd_nan_glm_speed_like_reference(cuda):
    """With the default initial_c_h = NaN the cleaning terms are NaN; the
    reference's @test_approx compares such arrays by NaN positions and the
    remaining values (test/test_macros.jl)."""
    semi, orc = _semi("ec", 2, 2, 3, False, c_h=float("nan"))
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    T.synchronize(semi)
    got, ref = du.cpu().numpy(), orc.rhs(u_host)
    assert np.isnan(ref).any()
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert_rel(got[ok], ref[ok], RTOL64, "non-NaN values")


@pytest.mark.parametrize("setup,d,level,p", [("ec", 2, 3, 3), ("shock", 3, 1, 4)])
def test_mhd_tiles_bit_identical(setup, d, level, p, cuda):
    """Every valid tile of the MHD kernels (at most 8 warps per block) gives
    the same bits."""
    semi, _ = _semi(setup, d, level, p, False)
    _, u = _u(semi, cuda)
    ref = cuda.empty_like(u)
    T.rhs_gpu(ref, u, semi, 0.0)
    seen = 0
    for w in range(1, 9):
        for g in (1, 2, 4):
            if w * g > 8:
                continue
            try:
                T.set_tile(semi, w, g)
            except T.TrixiError:
                continue
            du = cuda.empty_like(u)
            T.rhs_gpu(du, u, semi, 0.0)
            T.synchronize(semi)
            assert cuda.equal(du, ref), (w, g)
            seen += 1
    T.set_tile(semi, 0, 0)
    assert seen >= 2
    with pytest.raises(T.TrixiError):
        T.set_tile(semi, 8, 2)  # 16 warps: beyond the MHD kernels' 256-thread blocks


def test_mhd_rejections(cuda):
    """Combinations the MHD kernels do not cover fail loudly."""
    mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=2)
    eq = T.IdealGlmMhdEquations2D(1.4, 1.0)
    ic = T.initial_condition_weak_blast_wave
    # weak form
    with pytest.raises(T.TrixiError):
        T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, T.DGSEMGPU(
            polydeg=3, surface_flux=(T.flux_lax_friedrichs, T.flux_nonconservative_powell)))
    # plain fluxes for a system with nonconservative terms
    with pytest.raises(ValueError):
        T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, T.DGSEMGPU(
            polydeg=3, surface_flux=T.flux_lax_friedrichs,
            volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_hindenlang_gassner)))
    # polydeg 5 is not compiled for MHD
    with pytest.raises(T.TrixiError):
        T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, T.DGSEMGPU(
            polydeg=5, surface_flux=(T.flux_lax_friedrichs, T.flux_nonconservative_powell),
            volume_integral=T.VolumeIntegralFluxDifferencing((T.flux_hindenlang_gassner,
                                                              T.flux_nonconservative_powell))))


def _np_prim(eq, u):
    uu = u.reshape(-1, eq.nvariables).T
    rho, v, p = eq.cons2prim(uu)
    return uu, rho, v, p


def test_mhd_max_dt(cuda):
    """max_dt with |v_d| + the fast magnetosonic speed (StepsizeCallback)."""
    for d in (1, 2, 3):
        semi, _ = _semi("alfven", d, 3 if d < 3 else 2, 3, False)
        u_host, u = _u(semi, cuda)
        eq = semi.equations
        uu, rho, v, p = _np_prim(eq, u_host)
        a2, b2 = eq.gamma * p / rho, np.sum(uu[5:8] ** 2, axis=0) / rho
        E, NN = semi.nelements, semi.nnodes ** d
        lam = []
        for k in range(d):
            cf = np.sqrt(0.5 * (a2 + b2 + np.sqrt((a2 + b2) ** 2 - 4 * a2 * uu[5 + k] ** 2 / rho)))
            lam.append(np.max((np.abs(v[k]) + cf).reshape(E, NN), axis=1))
        m = np.max(semi.containers.inverse_jacobian * np.sum(lam, axis=0))
        ref = 2.0 / (semi.nnodes * m)
        assert abs(T.max_dt(u, semi) - ref) <= 1e-13 * ref


def test_mhd_integrals(cuda):
    """State and entropy integrals, and the entropy production of the
    entropy-conservative set-up (flux_hindenlang_gassner + Powell terms on a
    periodic mesh): zero to round-off, on the GPU's own rhs."""
    semi, _ = _semi("ec", 2, 3, 3, False)
    u_host, u = _u(semi, cuda)
    eq = semi.equations
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    w1 = semi.solver.basis.weights
    wn = np.multiply.outer(w1, w1).T.reshape(-1)
    J = (1.0 / semi.containers.inverse_jacobian) ** 2
    state = T.integrate(u, semi, "state")
    ref = np.einsum("e,n,env->v", J, wn, u_host.reshape(semi.nelements, -1, eq.nvariables))
    assert_rel(state, ref, 1e-13, "state integral")
    uu, rho, v, p = _np_prim(eq, u_host)
    s = np.log(p) - eq.gamma * np.log(rho)
    S = (-rho * s / (eq.gamma - 1)).reshape(semi.nelements, -1)
    assert_rel(T.integrate(u, semi, "entropy"), [np.einsum("e,n,en->", J, wn, S)], 1e-13, "entropy integral")
    prod = T.integrate(u, semi, "entropy_production", du=du)[0]
    scale = float(np.einsum("e,n,en->", J, wn, np.abs(S)))
    assert abs(prod) < 1e-11 * scale, (prod, scale)


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("kind", ["convergence_test", "weak_blast_wave"])
def test_mhd_gpu_initial_conditions_and_error_norms(d, kind, cuda):
    """compute_coefficients on the GPU for the MHD built-in initial conditions
    equals the host version; calc_error_norms of the exact state is zero and
    of a perturbed one matches numpy."""
    setup = "alfven" if kind == "convergence_test" else "ec"
    semi, _ = _semi(setup, d, 2 if d < 3 else 1, 3, False)
    host = semi.compute_coefficients_host(t=0.3 if kind == "convergence_test" else 0.0)
    u = T.compute_coefficients_gpu(semi, kind, t=0.3 if kind == "convergence_test" else 0.0)
    T.synchronize(semi)
    np.testing.assert_allclose(u.cpu().numpy(), host, rtol=1e-13, atol=1e-13)
    if kind == "convergence_test":
        # against the exact solution on 2N-1 analysis nodes: the interpolation
        # error of the degree-3 nodal state, small but nonzero (the coarse 3D
        # mesh, 2 elements per wavelength, shows ~5e-2); rho and E are exact
        l2, linf = T.calc_error_norms(u, semi, t=0.3, kind=kind)
        assert l2.shape == (semi.equations.nvariables,)
        assert 0 < np.max(l2) < 0.1 and np.max(linf) < 0.2
        assert l2[0] < 1e-14
        l2b, linfb = T.calc_error_norms(u, semi, u_ref=u)
        assert np.all(l2b == 0.0) and np.all(linfb == 0.0)


# ---------------------------------------------------------------------------
# Dirichlet boundaries: BoundaryConditionDirichlet on every side of a
# non-periodic TreeMesh with the MHD boundary functions; each boundary face
# adds 0.5 Phi(u_inner, u_boundary) on the element's side, as an interface
# face does on each of its sides.

def _bnd_semi(setup, d, level, polydeg=3, refined=False, precision="fp64", c_h=0.8):
    if setup == "alfven":
        gamma, ic = 5.0 / 3.0, T.initial_condition_convergence_test
        lo, hi = {1: (0.0, 1.0), 2: (0.0, np.sqrt(2.0)), 3: (-1.0, 1.0)}[d]
    else:
        gamma, ic = 1.4, T.initial_condition_weak_blast_wave
        lo, hi = (-1.0, 1.0)
    patches = [dict(type="box", coordinates_min=(lo,) * d,
                    coordinates_max=(lo + 0.5 * (hi - lo),) * d)] if refined else []
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches,
                      periodicity=False)
    eq = EQS[d](gamma, c_h)
    if setup == "shock":
        ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
        sflux = _pair(T.flux_hindenlang_gassner, d)
        vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=_pair(T.flux_hindenlang_gassner, d),
                                              volume_flux_fv=sflux)
    else:
        vf = T.flux_central if (setup == "alfven" and d == 2) else T.flux_hindenlang_gassner
        sflux, vi = _pair(T.flux_lax_friedrichs, d), T.VolumeIntegralFluxDifferencing(_pair(vf, d))
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=sflux, volume_integral=vi)
    bc = T.BoundaryConditionDirichlet(ic)
    bcs = dict(x_neg=bc, x_pos=bc, y_neg=bc, y_pos=bc, z_neg=bc, z_pos=bc)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, boundary_conditions=bcs, precision=precision)
    return semi, Oracle.from_semi(semi)


BND_CASES = [
    ("alfven", 1, 3, 3, False),
    ("alfven", 2, 3, 3, False),
    ("alfven", 2, 3, 3, True),      # mortars touching the boundary
    ("alfven", 3, 2, 3, False),
    ("blast", 3, 1, 3, True),
    ("shock", 2, 3, 4, False),
    ("shock", 3, 2, 3, False),
    ("blast", 2, 2, 2, False),
]


@pytest.mark.parametrize("case", BND_CASES, ids=[_ids(c) for c in BND_CASES])
def test_mhd_rhs_with_boundaries_matches_oracle(case, cuda):
    setup, d, level, p, refined = case
    semi, orc = _bnd_semi(setup, d, level, p, refined)
    assert semi.containers.nboundaries > 0
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.37)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host, 0.37), RTOL64, "mhd rhs with boundaries")


@pytest.mark.parametrize("case", [BND_CASES[2], BND_CASES[5]], ids=[_ids(c) for c in (BND_CASES[2], BND_CASES[5])])
def test_mhd_mixed_rhs_with_boundaries_close_to_oracle(case, cuda):
    setup, d, level, p, refined = case
    semi, orc = _bnd_semi(setup, d, level, p, refined, precision="mixed")
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.37)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host, 0.37), RTOL_MIXED, "mixed mhd rhs with boundaries")


@pytest.mark.parametrize("d", [1, 2, 3])
def test_mhd_boundary_stages_match_oracle(d, cuda):
    """cuda_prolong2boundaries! and cuda_boundary_flux! (with the Powell
    terms) one by one, then the whole staged rhs."""
    semi, orc = _bnd_semi("alfven", d, 2, 3, d == 2)
    u_host, u = _u(semi, cuda)
    T.cuda_prolong2boundaries(u, semi)
    T.synchronize(semi)
    bu = semi.container(T._lib.CONTAINER_BOUNDARIES_U).cpu().numpy()
    bu_ref = orc.prolong2boundaries(u_host)
    assert np.array_equal(bu, bu_ref)
    T.cuda_boundary_flux(0.25, semi)
    T.synchronize(semi)
    sfv = semi.container(T._lib.CONTAINER_SURFACE_FLUX_VALUES).cpu().numpy()
    sfv_ref = orc.boundary_flux(bu_ref, 0.25, np.zeros_like(sfv))
    nf = (semi.nnodes ** (d - 1)) * semi.equations.nvariables
    mask = np.zeros(sfv.size // nf, dtype=bool)
    c = semi.containers
    for e, side, o in zip(c.boundary_neighbor_ids, c.boundary_neighbor_sides, c.boundary_orientations):
        mask[(e - 1) * 2 * d + 2 * (o - 1) + (1 if side == 1 else 0)] = True
    assert_rel(sfv.reshape(-1, nf)[mask], sfv_ref.reshape(-1, nf)[mask], RTOL64, "mhd boundary flux")
    # the whole rhs stage by stage (volume, interfaces, boundaries, mortars,
    # surface integral, Jacobian), as rhs_gpu! calls them
    du = cuda.empty_like(u)
    T.cuda_volume_integral(du, u, semi)
    T.cuda_prolong2interfaces(u, semi)
    T.cuda_interface_flux(semi)
    T.cuda_prolong2boundaries(u, semi)
    T.cuda_boundary_flux(0.25, semi)
    T.cuda_prolong2mortars(u, semi)
    T.cuda_mortar_flux(semi)
    T.cuda_surface_integral(du, semi)
    T.cuda_jacobian(du, semi)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host, 0.25), RTOL64, "staged mhd rhs with boundaries")


@pytest.mark.parametrize("precision,rtol", [("fp64", RTOL64), ("mixed", RTOL_MIXED)])
def test_mhd_rk_steps_with_time_dependent_boundaries(precision, rtol, cuda):
    """The Alfven wave's boundary states follow the RK stage times."""
    semi, orc = _bnd_semi("alfven", 2, 3, 3, True, precision=precision)
    u_host, u = _u(semi, cuda)
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.1, 1e-3, 3, semi)
    T.synchronize(semi)
    uo, _ = orc.rk_ck2n54(u_host, 0.1, 1e-3, 3)
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, rtol * 10, "mhd rk increment")


def test_mhd_gpu_convergence_with_dirichlet_boundaries(cuda):
    """2D Alfven wave with its exact state on the boundary, FP64: errors at
    t = 0.1 on levels 2 and 3 fall at about polydeg + 1 = 4th order."""
    errs = []
    for level in (2, 3):
        semi, _ = _bnd_semi("alfven", 2, level, 3)
        x = semi.containers.node_coordinates.reshape(-1, 2).T
        u = cuda.from_numpy(np.ascontiguousarray(
            T.initial_condition_convergence_test(x, 0.0, semi.equations).T.reshape(semi.u_shape()))).to(semi.device)
        k = cuda.zeros_like(u)
        h = np.sqrt(2.0) / 2 ** level
        nsteps = int(np.ceil(0.1 / (0.5 * h / 4 / 2.0)))
        T.rk_steps(u, k, 0.0, 0.1 / nsteps, nsteps, semi)
        ue = T.initial_condition_convergence_test(x, 0.1, semi.equations).T.reshape(semi.u_shape())
        errs.append(float(np.sqrt(np.mean((u.cpu().numpy() - ue) ** 2))))
    assert np.log2(errs[0] / errs[1]) > 3.0, errs
