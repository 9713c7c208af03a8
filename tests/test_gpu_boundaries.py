"""Non-periodic meshes, Dirichlet boundaries and source terms on the GPU
(through the C ABI) against the CPU oracle.  Mirrors the reference's
test/tree_dgsem_{1,2,3}d/euler_source_terms_nonperiodic.jl set-up:
BoundaryConditionDirichlet(initial_condition_convergence_test) on every side,
source_terms_convergence_test, flux_lax_friedrichs surface flux; plus flux
differencing, shock capturing, mortars at the boundary and linear advection."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

RTOL64 = 1e-12
RTOL_MIXED = 5e-4


def _semi(eqname, d, level, polydeg=3, refined=False, vol="weak", sflux=None, bc=None, source=True,
          precision="fp64"):
    lo, hi = 0.0, 2.0
    patches = [dict(type="box", coordinates_min=(lo,) * d, coordinates_max=(1.0,) * d)] if refined else []
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches,
                      periodicity=False)
    if eqname == "adv":
        eq = {1: T.LinearScalarAdvectionEquation1D, 2: T.LinearScalarAdvectionEquation2D,
              3: T.LinearScalarAdvectionEquation3D}[d]((0.2, -0.7, 0.5)[:d] if d > 1 else (1.0,))
        source = False
    else:
        eq = {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
              3: T.CompressibleEulerEquations3D}[d](1.4)
    if vol == "weak":
        vi = T.VolumeIntegralWeakForm()
    elif vol == "fd":
        vi = T.VolumeIntegralFluxDifferencing(T.flux_ranocha if eqname != "adv" else T.flux_central)
    else:
        ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=True)
        vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=sflux or T.flux_lax_friedrichs, volume_integral=vi)
    ic = bc or T.initial_condition_convergence_test
    bcs = T.BoundaryConditionDirichlet(ic)
    bcs = dict(x_neg=bcs, x_pos=bcs, y_neg=bcs, y_pos=bcs, z_neg=bcs, z_pos=bcs)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, boundary_conditions=bcs,
                                             source_terms=T.source_terms_convergence_test if source else None,
                                             precision=precision)
    return semi, Oracle.from_semi(semi)


def _u(semi, cuda, t=0.0):
    x = semi.containers.node_coordinates.reshape(-1, semi.mesh.ndims).T
    u = semi.initial_condition(x, t, semi.equations).T.reshape(semi.u_shape())
    # a perturbation so that interior and boundary states differ
    rng = np.random.default_rng(7)
    u = np.ascontiguousarray(u * (1.0 + 0.01 * rng.standard_normal(u.shape)))
    return u, cuda.from_numpy(u).to(semi.device)


CASES = [
    ("euler", 1, 3, 3, False, "weak", {}),
    ("euler", 2, 3, 3, False, "weak", {}),
    ("euler", 3, 2, 3, False, "weak", {}),
    ("euler", 2, 3, 3, True, "weak", {}),                      # mortars touching the boundary
    ("euler", 2, 3, 3, False, "fd", {}),
    ("euler", 3, 2, 3, True, "fd", dict(sflux=T.flux_ranocha)),
    ("euler", 2, 2, 2, False, "fd", {}),
    ("euler", 2, 2, 5, False, "weak", {}),
    ("euler", 2, 3, 3, False, "sc", dict(bc=T.initial_condition_weak_blast_wave, source=False)),
    ("adv", 2, 3, 3, False, "weak", {}),
    ("adv", 3, 2, 3, True, "weak", {}),
    ("adv", 1, 4, 3, False, "weak", {}),
]


def _ids(c):
    return f"{c[0]}-{c[1]}d-L{c[2]}-p{c[3]}{'-ref' if c[4] else ''}-{c[5]}{'-' + '-'.join(sorted(c[6])) if c[6] else ''}"


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_rhs_with_boundaries_matches_oracle(case, cuda):
    eqname, d, level, p, refined, vol, extra = case
    semi, orc = _semi(eqname, d, level, p, refined, vol, **extra)
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.37)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host, 0.37), RTOL64, "rhs")


@pytest.mark.parametrize("case", [CASES[1], CASES[5], CASES[9]], ids=[_ids(c) for c in (CASES[1], CASES[5], CASES[9])])
def test_mixed_rhs_with_boundaries_close_to_oracle(case, cuda):
    eqname, d, level, p, refined, vol, extra = case
    semi, orc = _semi(eqname, d, level, p, refined, vol, precision="mixed", **extra)
    u_host, u = _u(semi, cuda)
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.37)
    T.synchronize(semi)
    assert_rel(du.cpu().numpy(), orc.rhs(u_host, 0.37), RTOL_MIXED, "mixed rhs")


@pytest.mark.parametrize("d", [1, 2, 3])
def test_boundary_stages_match_oracle(d, cuda):
    """cuda_prolong2boundaries! / cuda_boundary_flux! / cuda_sources! one by one,
    as the reference's stage tests do."""
    semi, orc = _semi("euler", d, 2, 3, False, "weak")
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
    mask = np.zeros(sfv.size // nf, dtype=bool)  # (element, direction) slots of boundary faces
    c = semi.containers
    for e, side, o in zip(c.boundary_neighbor_ids, c.boundary_neighbor_sides, c.boundary_orientations):
        mask[(e - 1) * 2 * d + 2 * (o - 1) + (1 if side == 1 else 0)] = True
    got = sfv.reshape(-1, nf)[mask]
    ref = sfv_ref.reshape(-1, nf)[mask]
    assert_rel(got, ref, RTOL64, "boundary flux")
    du = cuda.zeros_like(u)
    T.cuda_sources(du, u, 0.25, semi)
    T.synchronize(semi)
    du_ref = orc.sources(np.zeros(du.numel()), 0.25)
    np.testing.assert_allclose(du.cpu().numpy().reshape(-1), du_ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("precision,rtol", [("fp64", RTOL64), ("mixed", RTOL_MIXED)])
def test_rk_steps_with_time_dependent_boundaries(precision, rtol, cuda):
    """Boundary states and sources follow the RK stage times t + c_s dt."""
    semi, orc = _semi("euler", 2, 3, 3, False, "fd", precision=precision)
    u_host, u = _u(semi, cuda)
    k = cuda.zeros_like(u)
    T.rk_steps(u, k, 0.1, 2e-3, 3, semi)
    T.synchronize(semi)
    uo, ko = u_host.copy(), np.zeros_like(u_host)
    import ctypes as C
    pd = C.POINTER(C.c_double)
    orc.lib.oracle_rk_ck2n54(orc._h, uo.ctypes.data_as(pd), ko.ctypes.data_as(pd), 0.1, 2e-3, 3)
    # compare the change of the state (the state itself is O(1))
    assert_rel(u.cpu().numpy() - u_host, uo - u_host, rtol * 10, "rk increment")


def test_gpu_convergence_order(cuda):
    """2D Euler convergence test with Dirichlet boundaries and sources:
    errors after t = 0.1 on levels 3 and 4 fall at ~4th order (polydeg 3)."""
    errs = []
    for level in (3, 4):
        semi, _ = _semi("euler", 2, level, 3, False, "fd")
        x = semi.containers.node_coordinates.reshape(-1, 2).T
        u = cuda.from_numpy(np.ascontiguousarray(
            T.initial_condition_convergence_test(x, 0.0, semi.equations).T.reshape(semi.u_shape()))).to(semi.device)
        k = cuda.zeros_like(u)
        h = 2.0 / 2 ** level
        nsteps = int(np.ceil(0.1 / (0.4 * h / 4 / 3.0)))
        T.rk_steps(u, k, 0.0, 0.1 / nsteps, nsteps, semi)
        ue = T.initial_condition_convergence_test(x, 0.1, semi.equations).T.reshape(semi.u_shape())
        errs.append(float(np.sqrt(np.mean((u.cpu().numpy() - ue) ** 2))))
    assert np.log2(errs[0] / errs[1]) > 3.5, errs
