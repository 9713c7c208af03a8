"""Ideal GLM-MHD in the CPU oracle (no GPU): IdealGlmMhdEquations{1,2,3}D
with flux_hindenlang_gassner / flux_central / flux_lax_friedrichs paired with
flux_nonconservative_powell, as the reference's MHD tests set them up
(test/tree_dgsem_2d/mhd_ec.jl, mhd_alfven_wave.jl, mhd_alfven_wave_mortar.jl,
mhd_shock.jl and their 1D/3D versions).  Parity with Trixi.jl is unpinned
(no golden vectors); these pins are properties of the discretization:
free-stream preservation (which also checks the signs and factors 1/2 of the
nonconservative volume, surface, mortar and FV terms), discrete entropy
conservation of the Hindenlang-Gassner flux with the Powell terms, and the
convergence order on the smooth Alfven waves."""
import ctypes as C

import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import (FLUX_CENTRAL, FLUX_HINDENLANG_GASSNER, FLUX_HLLE, FLUX_LLF, NONCONS_NONE, NONCONS_POWELL,
                           VOL_FLUXDIFF, VOL_SHOCK_HG, Oracle, basis)

MHD = {1: T.IdealGlmMhdEquations1D, 2: T.IdealGlmMhdEquations2D, 3: T.IdealGlmMhdEquations3D}


def _oracle(d, level, polydeg=3, lo=-2.0, hi=2.0, refined=False, vflux=FLUX_HINDENLANG_GASSNER,
            sflux=FLUX_HINDENLANG_GASSNER, vol=VOL_FLUXDIFF, gamma=1.4, c_h=0.8):
    patches = [dict(type="box", coordinates_min=(lo,) * d, coordinates_max=(0.5 * (lo + hi),) * d)] if refined else []
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches)
    cont = mesh.build_containers(basis(polydeg)["nodes"])
    eq = MHD[d](gamma, c_h)
    orc = Oracle(cont, d, polydeg, eq.nvariables, eq.code, gamma=gamma, volume_integral=vol, volume_flux=vflux,
                 surface_flux=sflux, volume_flux_fv=sflux,
                 nonconservative_flux=NONCONS_POWELL if d > 1 else NONCONS_NONE, glm_speed=c_h)
    return eq, cont, orc


def _state(eq, cont, ic):
    d = eq.ndims
    x = cont.node_coordinates.reshape(-1, d).T
    n = round(cont.node_coordinates.size / (d * cont.nelements))
    shape = (cont.nelements, n, eq.nvariables)
    return np.ascontiguousarray(ic(x, 0.0, eq).T.reshape(shape))


def _smooth(x, t, eq, seed=3):
    """A smooth periodic state on [-2, 2]^d with all nine fields varying."""
    rng = np.random.default_rng(seed)
    d, n = eq.ndims, x.shape[1]
    ph = [rng.uniform(0, 2 * np.pi, size=d) for _ in range(9)]
    f = lambda i, a: a * np.prod([np.sin(0.5 * np.pi * x[k] + ph[i][k]) for k in range(d)], axis=0)  # noqa: E731
    rho = 1.0 + f(0, 0.2)
    v = np.stack([0.1 + f(1, 0.1), -0.05 + f(2, 0.1), f(3, 0.1)])
    p = 1.0 + f(4, 0.2)
    B = np.stack([0.5 + f(5, 0.2), -0.3 + f(6, 0.2), 0.2 + f(7, 0.2)])
    psi = f(8, 0.05)
    return eq.prim2cons(rho, v, p, B, psi)


def _entropy_vars(eq, u):
    """Entropy variables of ideal GLM-MHD for S = -rho s/(gamma-1),
    s = ln p - gamma ln rho (Derigs et al. 2018): ((gamma-s)/(gamma-1) -
    beta|v|^2, 2 beta v, -2 beta, 2 beta B, 2 beta psi), beta = rho/(2p)."""
    g = eq.gamma
    uu = u.reshape(-1, eq.nvariables).T
    rho, v, p = eq.cons2prim(uu)
    s = np.log(p) - g * np.log(rho)
    beta = 0.5 * rho / p
    w = np.empty_like(uu)
    w[0] = (g - s) / (g - 1) - beta * np.sum(v * v, axis=0)
    w[1:4] = 2 * beta * v
    w[4] = -2 * beta
    w[5:8] = 2 * beta * uu[5:8]
    if eq.nvariables == 9:
        w[8] = 2 * beta * uu[8]
    return w.T.reshape(u.shape)


def _weights(cont, d, polydeg):
    w1 = basis(polydeg)["weights"]
    wn = w1
    for _ in range(d - 1):
        wn = np.multiply.outer(wn, w1)
    # node order: first coordinate fastest
    return np.ascontiguousarray(wn.T).reshape(-1)


@pytest.mark.parametrize("d,level,vflux,sflux,vol,refined", [
    (1, 3, FLUX_HINDENLANG_GASSNER, FLUX_LLF, VOL_FLUXDIFF, False),
    (2, 2, FLUX_HINDENLANG_GASSNER, FLUX_HINDENLANG_GASSNER, VOL_FLUXDIFF, False),
    (2, 2, FLUX_CENTRAL, FLUX_LLF, VOL_FLUXDIFF, False),
    (2, 2, FLUX_HINDENLANG_GASSNER, FLUX_LLF, VOL_FLUXDIFF, True),
    (2, 2, FLUX_HINDENLANG_GASSNER, FLUX_HINDENLANG_GASSNER, VOL_SHOCK_HG, True),
    (3, 1, FLUX_HINDENLANG_GASSNER, FLUX_LLF, VOL_FLUXDIFF, True),
    (3, 1, FLUX_HINDENLANG_GASSNER, FLUX_HINDENLANG_GASSNER, VOL_SHOCK_HG, False),
    (1, 3, FLUX_HINDENLANG_GASSNER, FLUX_HLLE, VOL_FLUXDIFF, False),
    (2, 2, FLUX_HINDENLANG_GASSNER, FLUX_HLLE, VOL_FLUXDIFF, True),    # mhd_alfven_wave_mortar.jl
    (2, 2, FLUX_HINDENLANG_GASSNER, FLUX_HLLE, VOL_SHOCK_HG, True),
    (3, 1, FLUX_HINDENLANG_GASSNER, FLUX_HLLE, VOL_FLUXDIFF, True),
])
def test_mhd_free_stream(d, level, vflux, sflux, vol, refined):
    """A constant state (with a magnetic field and psi) is preserved to
    round-off: the conservative fluxes are consistent and the
    nonconservative volume, interface, mortar and FV-subcell terms cancel."""
    eq, cont, orc = _oracle(d, level, refined=refined, vflux=vflux, sflux=sflux, vol=vol)
    state = eq.prim2cons(np.array([1.3]), np.array([[0.2], [-0.1], [0.3]]), np.array([0.9]),
                         np.array([[0.7], [-0.4], [0.5]]), np.array([0.1]))[:, 0]
    n = (4,) * d
    u = np.broadcast_to(state, (cont.nelements,) + (int(np.prod(n)),) + (eq.nvariables,)).copy()
    # shock capturing blends in the FV part where the indicator fires; force it on
    du = orc.rhs(u, 0.0) if vol != VOL_SHOCK_HG else None
    if vol == VOL_SHOCK_HG:
        alpha = np.full(cont.nelements, 0.4)
        du = orc.volume_integral(u, alpha)
        iu = orc.prolong2interfaces(u)
        sfv = orc.interface_flux(iu)
        if cont.nmortars:
            orc.mortar_flux(orc.prolong2mortars(u), sfv)
        du = orc.jacobian(orc.surface_integral(du, sfv))
    assert np.max(np.abs(du)) < 1e-12, np.max(np.abs(du))


@pytest.mark.parametrize("d,level", [(2, 2), (3, 1)])
@pytest.mark.parametrize("c_h", [0.0, 0.8])
def test_mhd_entropy_conservation(d, level, c_h):
    """flux_hindenlang_gassner in the volume and on the surfaces, with
    flux_nonconservative_powell, conserves the total entropy on a periodic
    mesh: sum_e J_e sum_i w_i v(u_i) . du_i = 0 up to round-off."""
    eq, cont, orc = _oracle(d, level, c_h=c_h)
    u = _state(eq, cont, _smooth)
    # a node-wise perturbation: traces jump across every interface
    u *= 1.0 + 0.01 * np.random.default_rng(11).standard_normal(u.shape)
    du = orc.rhs(u, 0.0)
    v = _entropy_vars(eq, u)
    w = _weights(cont, d, 3)
    J = 1.0 / cont.inverse_jacobian
    terms = J[:, None] * w[None, :] * np.sum(v * du, axis=2)
    total, scale = float(np.sum(terms)), float(np.sum(np.abs(terms)))
    assert abs(total) <= 1e-12 * scale, (total, scale)
    # the LLF surface flux dissipates entropy instead
    _, _, orc2 = _oracle(d, level, c_h=c_h, sflux=FLUX_LLF)
    du2 = orc2.rhs(u, 0.0)
    assert float(np.sum(J[:, None] * w[None, :] * np.sum(v * du2, axis=2))) < -1e-8 * scale


def _alfven_error(d, level, t_end=0.1, polydeg=3, vflux=FLUX_CENTRAL, sflux=FLUX_LLF):
    lo, hi = (0.0, 1.0) if d == 1 else ((0.0, np.sqrt(2.0)) if d == 2 else (-1.0, 1.0))
    eq, cont, orc = _oracle(d, level, polydeg=polydeg, lo=lo, hi=hi, vflux=vflux, sflux=sflux,
                            gamma=5.0 / 3.0, c_h=1.0)
    u = _state(eq, cont, T.initial_condition_convergence_test)
    h = (hi - lo) / 2 ** level
    nsteps = int(np.ceil(t_end / (0.3 * h / (polydeg + 1) / 2.0)))
    k = np.zeros_like(u)
    pd = C.POINTER(C.c_double)
    orc.lib.oracle_rk_ck2n54(orc._h, u.ctypes.data_as(pd), k.ctypes.data_as(pd), 0.0, t_end / nsteps, nsteps)
    x = cont.node_coordinates.reshape(-1, d).T
    ue = T.initial_condition_convergence_test(x, t_end, eq).T.reshape(u.shape)
    return float(np.sqrt(np.mean((u - ue) ** 2)))


@pytest.mark.parametrize("d,levels,vflux,sflux,min_eoc", [
    (1, (2, 3), FLUX_HINDENLANG_GASSNER, FLUX_LLF, 3.5),
    (2, (2, 3), FLUX_CENTRAL, FLUX_LLF, 3.0),
    (2, (2, 3), FLUX_HINDENLANG_GASSNER, FLUX_LLF, 3.0),
    (1, (2, 3), FLUX_HINDENLANG_GASSNER, FLUX_HLLE, 3.5),
    (2, (2, 3), FLUX_HINDENLANG_GASSNER, FLUX_HLLE, 3.0),
])
def test_mhd_alfven_wave_convergence(d, levels, vflux, sflux, min_eoc):
    """The smooth Alfven waves converge at about polydeg + 1 (polydeg 3;
    measured 3.2-3.7 between these coarse levels, still pre-asymptotic)."""
    e0, e1 = (_alfven_error(d, lv, vflux=vflux, sflux=sflux) for lv in levels)
    assert np.log2(e0 / e1) > min_eoc, (e0, e1)


def test_mhd_nan_glm_speed_propagates():
    """Trixi's default initial_c_h is NaN until a GlmSpeedCallback sets it;
    the cleaning terms then carry NaN into the result (the reference's
    @test_approx compares such arrays NaN-position-wise)."""
    eq, cont, orc = _oracle(2, 1, c_h=float("nan"))
    u = _state(eq, cont, _smooth)
    du = orc.rhs(u, 0.0)
    assert np.isnan(du).any()
    # with c_h = 0 everything is finite
    _, _, orc0 = _oracle(2, 1, c_h=0.0)
    assert np.all(np.isfinite(orc0.rhs(u, 0.0)))


# ---------------------------------------------------------------------------
# Dirichlet boundaries (BoundaryConditionDirichlet on every side of a
# non-periodic TreeMesh, as the reference's euler_source_terms_nonperiodic.jl
# set-ups use them), here with the MHD boundary functions and the Powell
# terms on the element's side of each boundary face.

def _bnd_oracle(d, level, lo, hi, bc, bc_params=None, polydeg=3, periodic=False, gamma=5.0 / 3.0, c_h=0.8,
                vflux=FLUX_HINDENLANG_GASSNER, sflux=FLUX_LLF):
    mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, periodicity=periodic)
    cont = mesh.build_containers(basis(polydeg)["nodes"])
    eq = MHD[d](gamma, c_h)
    orc = Oracle(cont, d, polydeg, eq.nvariables, eq.code, gamma=gamma, volume_integral=VOL_FLUXDIFF,
                 volume_flux=vflux, surface_flux=sflux, volume_flux_fv=sflux,
                 nonconservative_flux=NONCONS_POWELL if d > 1 else NONCONS_NONE, glm_speed=c_h,
                 boundary_function=-1 if periodic else bc, boundary_params=bc_params)
    return eq, cont, orc


@pytest.mark.parametrize("d", [1, 2, 3])
@pytest.mark.parametrize("kind,ic", [(1, T.initial_condition_convergence_test), (2, T.initial_condition_weak_blast_wave)])
def test_oracle_mhd_boundary_states_match_host(d, kind, ic):
    """The oracle's MHD boundary functions (Alfven waves, weak blast wave in
    B = (1, 1, 1)) equal the host initial conditions the GPU tests use."""
    lo, hi = {1: (0.0, 1.0), 2: (0.0, np.sqrt(2.0)), 3: (-1.0, 1.0)}[d] if kind == 1 else (-1.0, 1.0)
    eq, cont, orc = _bnd_oracle(d, 1, lo, hi, kind)
    x = np.ascontiguousarray(cont.node_coordinates.reshape(-1, d))
    pd = C.POINTER(C.c_double)
    for t in (0.0, 0.3):
        got = np.empty((x.shape[0], eq.nvariables))
        for i in range(x.shape[0]):
            orc.lib.oracle_eval_ic(orc._h, kind, None, x[i].ctypes.data_as(pd), t, got[i].ctypes.data_as(pd))
        np.testing.assert_allclose(got, ic(x.T, t, eq).T, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_mhd_free_stream_with_dirichlet_boundaries(d):
    """A uniform magnetised state stays put with Dirichlet boundaries that
    hold it: in 1D a constant boundary state; in 2D/3D the weak blast
    wave's outer state (rho = p = 1, v = 0, B = (1, 1, 1)) on [1, 3]^d,
    which lies outside its blast radius."""
    if d == 1:
        eq = MHD[1](1.4, 0.8)
        state = eq.prim2cons(np.array([1.2]), np.array([[0.3], [-0.2], [0.1]]), np.array([0.9]),
                             np.array([[0.7], [0.4], [-0.5]]), None)[:, 0]
        eq, cont, orc = _bnd_oracle(1, 3, 0.0, 1.0, 0, state, gamma=1.4)
    else:
        eq, cont, orc = _bnd_oracle(d, 2, 1.0, 3.0, 2, gamma=1.4)
        state = eq.prim2cons(np.array([1.0]), np.zeros((3, 1)), np.array([1.0]), np.ones((3, 1)),
                             np.zeros(1))[:, 0]
    u = np.broadcast_to(state, (cont.nelements,) + (4,) * d + (eq.nvariables,)).copy()
    assert np.max(np.abs(orc.rhs(u, 0.0))) < 1e-12


@pytest.mark.parametrize("d", [2, 3])
def test_mhd_dirichlet_interior_equals_periodic(d):
    """With the exact Alfven wave as the boundary state, elements away from
    the boundary see the same neighbours as on the periodic mesh: their rhs
    is bit-identical.  The LGL nodes include the faces, so the periodic
    neighbour's trace is the exact state at the face node too: boundary
    elements differ by rounding only (the coordinates of the periodic image),
    Powell terms included -- the boundary takes 0.5 Phi(u_inner, u_boundary)
    as the interface takes 0.5 Phi(u_own, u_other)."""
    lo, hi = (0.0, np.sqrt(2.0)) if d == 2 else (-1.0, 1.0)
    level = 3 if d == 2 else 2
    eq, cont, orc_b = _bnd_oracle(d, level, lo, hi, 1)
    _, cont_p, orc_p = _bnd_oracle(d, level, lo, hi, 1, periodic=True)
    assert np.array_equal(cont.node_coordinates, cont_p.node_coordinates)
    x = cont.node_coordinates.reshape(-1, d).T
    u = np.ascontiguousarray(T.initial_condition_convergence_test(x, 0.0, eq).T.reshape(
        (cont.nelements, 4 ** d, eq.nvariables)))
    du_b, du_p = orc_b.rhs(u, 0.0), orc_p.rhs(u, 0.0)
    on_bnd = np.zeros(cont.nelements, dtype=bool)
    on_bnd[cont.boundary_neighbor_ids - 1] = True
    assert on_bnd.any() and not on_bnd.all()
    assert np.array_equal(du_b[~on_bnd], du_p[~on_bnd])
    diff = np.linalg.norm(du_b[on_bnd] - du_p[on_bnd]) / np.linalg.norm(du_p[on_bnd])
    assert diff < 1e-13, diff


def test_mhd_alfven_convergence_with_dirichlet_boundaries():
    """1D Alfven wave with its exact state on both ends: errors at t = 0.2
    on levels 3 and 4 fall at about polydeg + 1 = 4th order."""
    errs = []
    for level in (3, 4):
        eq, cont, orc = _bnd_oracle(1, level, 0.0, 1.0, 1, sflux=FLUX_LLF)
        x = cont.node_coordinates.reshape(-1, 1).T
        shape = (cont.nelements, 4, eq.nvariables)
        u = np.ascontiguousarray(T.initial_condition_convergence_test(x, 0.0, eq).T.reshape(shape))
        h = 1.0 / 2 ** level
        nsteps = int(np.ceil(0.2 / (0.5 * h / 4 / 2.0)))
        u, _ = orc.rk_ck2n54(u, 0.0, 0.2 / nsteps, nsteps)
        ue = T.initial_condition_convergence_test(x, 0.2, eq).T.reshape(shape)
        errs.append(float(np.sqrt(np.mean((u - ue) ** 2))))
    assert np.log2(errs[0] / errs[1]) > 3.5, errs
