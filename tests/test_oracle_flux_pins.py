"""Pointwise pins of the oracle's two-point fluxes on random states (no
GPU): consistency f#(u, u) = f(u) of every flux, symmetry of the symmetric
ones, Tadmor's entropy-conservation condition (w_r - w_l) . f* = psi_r -
psi_l for flux_ranocha (w the entropy variables, psi = rho v_o the entropy
flux potential), Phi(u, u) = phi(u) B_o(u) of the Powell term, and
flux_hlle against a numpy restatement of Einfeldt's signal speeds."""
import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import (EQ_ADVECTION, EQ_EULER, EQ_MHD, FLUX_CENTRAL, FLUX_HINDENLANG_GASSNER, FLUX_HLL,
                           FLUX_HLLE, FLUX_LLF, FLUX_LLF_NAIVE, FLUX_RANOCHA, FLUX_SHIMA_ETAL, NONCONS_NONE, NONCONS_POWELL,
                           Oracle, basis)


def _oracle(eq_code, d, nv, noncons=NONCONS_NONE, gamma=1.4, c_h=0.7):
    mesh = T.TreeMesh((-1.0,) * d, (1.0,) * d, initial_refinement_level=1)
    cont = mesh.build_containers(basis(2)["nodes"])
    return Oracle(cont, d, 2, nv, eq_code, gamma=gamma, advection_velocity=(0.3, -0.6, 0.9)[:d],
                  nonconservative_flux=noncons, glm_speed=c_h)


def _euler_state(rng, d, gamma=1.4):
    rho, p = rng.uniform(0.5, 2.0), rng.uniform(0.5, 2.0)
    v = rng.uniform(-1, 1, d)
    return np.concatenate([[rho], rho * v, [p / (gamma - 1) + 0.5 * rho * v @ v]])


def _mhd_state(rng, d, gamma=1.4):
    rho, p = rng.uniform(0.5, 2.0), rng.uniform(0.5, 2.0)
    v, B = rng.uniform(-1, 1, 3), rng.uniform(-1, 1, 3)
    psi = rng.uniform(-0.3, 0.3) if d > 1 else 0.0
    u = [rho, *(rho * v), p / (gamma - 1) + 0.5 * rho * v @ v + 0.5 * B @ B + 0.5 * psi * psi, *B]
    return np.array(u + ([psi] if d > 1 else []))


SYSTEMS = [("adv", d) for d in (1, 2, 3)] + [("euler", d) for d in (1, 2, 3)] + [("mhd", d) for d in (1, 2, 3)]
KINDS = {"adv": [FLUX_CENTRAL, FLUX_LLF, FLUX_LLF_NAIVE, FLUX_HLL],
         "euler": [FLUX_CENTRAL, FLUX_RANOCHA, FLUX_SHIMA_ETAL, FLUX_LLF, FLUX_LLF_NAIVE, FLUX_HLL, FLUX_HLLE],
         "mhd": [FLUX_CENTRAL, FLUX_HINDENLANG_GASSNER, FLUX_LLF, FLUX_LLF_NAIVE, FLUX_HLL, FLUX_HLLE]}
SYMMETRIC = {FLUX_CENTRAL, FLUX_RANOCHA, FLUX_SHIMA_ETAL, FLUX_HINDENLANG_GASSNER}


def _make(system, d):
    if system == "adv":
        return _oracle(EQ_ADVECTION, d, 1), (lambda rng: rng.uniform(-2, 2, 1))
    if system == "euler":
        return _oracle(EQ_EULER, d, d + 2), (lambda rng: _euler_state(rng, d))
    return (_oracle(EQ_MHD, d, 8 if d == 1 else 9, NONCONS_POWELL if d > 1 else NONCONS_NONE),
            (lambda rng: _mhd_state(rng, d)))


@pytest.mark.parametrize("system,d", SYSTEMS, ids=[f"{s}-{d}d" for s, d in SYSTEMS])
def test_consistency_and_symmetry(system, d):
    orc, state = _make(system, d)
    rng = np.random.default_rng(17)
    for _ in range(20):
        ul, ur = state(rng), state(rng)
        for o in range(d):
            f = orc.physical_flux(ul, o)
            for kind in KINDS[system]:
                fc = orc.two_point_flux(kind, ul, ul, o)
                np.testing.assert_allclose(fc, f, rtol=1e-13, atol=1e-13, err_msg=f"consistency kind {kind}")
                if kind in SYMMETRIC:
                    np.testing.assert_allclose(orc.two_point_flux(kind, ul, ur, o), orc.two_point_flux(kind, ur, ul, o),
                                               rtol=1e-13, atol=1e-13, err_msg=f"symmetry kind {kind}")


@pytest.mark.parametrize("d", [1, 2, 3])
def test_ranocha_entropy_conservation_condition(d):
    """(w_r - w_l) . f_ranocha = (rho v_o)_r - (rho v_o)_l (Tadmor 1987)."""
    g = 1.4
    orc = _oracle(EQ_EULER, d, d + 2, gamma=g)
    rng = np.random.default_rng(5)

    def entropy_vars(u):
        rho, m, E = u[0], u[1:1 + d], u[-1]
        v = m / rho
        p = (g - 1) * (E - 0.5 * rho * v @ v)
        s = np.log(p) - g * np.log(rho)
        return np.concatenate([[(g - s) / (g - 1) - 0.5 * rho / p * v @ v], rho / p * v, [-rho / p]])

    for _ in range(30):
        ul, ur = _euler_state(rng, d), _euler_state(rng, d)
        for o in range(d):
            f = orc.two_point_flux(FLUX_RANOCHA, ul, ur, o)
            lhs = (entropy_vars(ur) - entropy_vars(ul)) @ f
            rhs = ur[1 + o] - ul[1 + o]
            assert abs(lhs - rhs) <= 1e-12 * (1 + abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("d", [2, 3])
def test_powell_term_is_local_times_other(d):
    """Phi(u_l, u_r) = phi_P(u_l) B_o(u_r) + v_o(u_l) phi_GLM(u_l) psi(u_r)."""
    orc = _oracle(EQ_MHD, d, 9, NONCONS_POWELL)
    rng = np.random.default_rng(8)
    for _ in range(10):
        ul, ur = _mhd_state(rng, d), _mhd_state(rng, d)
        rho = ul[0]
        v, B, psi = ul[1:4] / rho, ul[5:8], ul[8]
        for o in range(d):
            Bo, psir = ur[5 + o], ur[8]
            expect = np.concatenate([[0.0], B * Bo, [v @ B * Bo + v[o] * psi * psir], v * Bo, [v[o] * psir]])
            np.testing.assert_allclose(orc.noncons_flux(ul, ur, o), expect, rtol=1e-14, atol=1e-14)


def _hll(fl, fr, ul, ur, lmin, lmax):
    if lmin >= 0:
        return fl
    if lmax <= 0:
        return fr
    return (lmax * fl - lmin * fr + lmin * lmax * (ur - ul)) / (lmax - lmin)


def _einfeldt_euler(ul, ur, o, d, g):
    """Einfeldt, Munz, Roe, Sjogreen (1991): Roe-averaged sound speed, the
    states' sound speeds times beta = sqrt((g-1)/(2g)), bounds around 0."""
    def prim(u):
        rho = u[0]
        v = u[1:1 + d] / rho
        p = (g - 1) * (u[-1] - 0.5 * rho * v @ v)
        return rho, v, p, (u[-1] + p) / rho, np.sqrt(g * p / rho)
    rl, vl, pl, hl, cl = prim(ul)
    rr, vr, pr, hr, cr = prim(ur)
    wl, wr = np.sqrt(rl) / (np.sqrt(rl) + np.sqrt(rr)), np.sqrt(rr) / (np.sqrt(rl) + np.sqrt(rr))
    v, h = wl * vl + wr * vr, wl * hl + wr * hr
    c = np.sqrt((g - 1) * (h - 0.5 * v @ v))
    beta = np.sqrt(0.5 * (g - 1) / g)
    return min(v[o] - c, vl[o] - beta * cl, 0.0), max(v[o] + c, vr[o] + beta * cr, 0.0)


def _mhd_prim(u, g):
    rho = u[0]
    v, B = u[1:4] / rho, u[5:8]
    psi = u[8] if u.size == 9 else 0.0
    p = (g - 1) * (u[4] - 0.5 * rho * v @ v - 0.5 * B @ B - 0.5 * psi * psi)
    return rho, v, B, p


def _fast(u, o, g):
    rho, v, B, p = _mhd_prim(u, g)
    a2, b2, bo2 = g * p / rho, B @ B / rho, B[o] ** 2 / rho
    return np.sqrt(0.5 * (a2 + b2 + np.sqrt((a2 + b2) ** 2 - 4 * a2 * bo2)))


def _roe_fast_mhd(ul, ur, o, g):
    """Cargo and Gallice (1997): the fast speed of the Roe-type average."""
    rl, vl, Bl, pl = _mhd_prim(ul, g)
    rr, vr, Br, pr = _mhd_prim(ur, g)
    sl, sr = np.sqrt(rl), np.sqrt(rr)
    v = (sl * vl + sr * vr) / (sl + sr)
    B = (sr * Bl + sl * Br) / (sl + sr)
    hl, hr = (ul[4] + pl + 0.5 * Bl @ Bl) / rl, (ur[4] + pr + 0.5 * Br @ Br) / rr
    h = (sl * hl + sr * hr) / (sl + sr)
    X = 0.5 * (Bl - Br) @ (Bl - Br) / (sl + sr) ** 2
    b2 = B @ B / (sl * sr)
    a2 = (2 - g) * X + (g - 1) * (h - 0.5 * v @ v - b2)
    return v[o], np.sqrt(0.5 * (a2 + b2 + np.sqrt((a2 + b2) ** 2 - 4 * a2 * B[o] ** 2 / (sl * sr))))


@pytest.mark.parametrize("system,d", [("euler", d) for d in (1, 2, 3)] + [("mhd", d) for d in (1, 2, 3)])
def test_hlle_matches_numpy_restatement(system, d):
    orc, state = _make(system, d)
    rng = np.random.default_rng(23)
    g = 1.4
    for _ in range(30):
        ul, ur = state(rng), state(rng)
        for o in range(d):
            if system == "euler":
                lmin, lmax = _einfeldt_euler(ul, ur, o, d, g)
            else:
                vo, cf = _roe_fast_mhd(ul, ur, o, g)
                lmin = min(ul[1 + o] / ul[0] - _fast(ul, o, g), vo - cf)
                lmax = max(ur[1 + o] / ur[0] + _fast(ur, o, g), vo + cf)
            ref = _hll(orc.physical_flux(ul, o), orc.physical_flux(ur, o), ul, ur, lmin, lmax)
            np.testing.assert_allclose(orc.two_point_flux(FLUX_HLLE, ul, ur, o), ref, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_mhd_roe_fast_speed_of_equal_states(d):
    """Without psi, the Roe-type average of two equal states is the state
    itself and its fast speed the state's fast magnetosonic speed."""
    rng = np.random.default_rng(4)
    for _ in range(10):
        u = _mhd_state(rng, 1)
        for o in range(d):
            vo, cf = _roe_fast_mhd(u, u, o, 1.4)
            assert np.isclose(vo, u[1 + o] / u[0], rtol=1e-14) and np.isclose(cf, _fast(u, o, 1.4), rtol=1e-13)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_euler_hlle_mirror_symmetry(d):
    """Reflecting x_o -> -x_o (v_o -> -v_o) and swapping the states negates
    the mass, energy and transverse-momentum fluxes and keeps the normal
    momentum flux: the Einfeldt bounds map onto each other."""
    orc, state = _make("euler", d)
    rng = np.random.default_rng(31)
    for _ in range(20):
        ul, ur = state(rng), state(rng)
        for o in range(d):
            m = np.ones(d + 2)
            m[1 + o] = -1.0
            f = orc.two_point_flux(FLUX_HLLE, ul, ur, o)
            fm = orc.two_point_flux(FLUX_HLLE, m * ur, m * ul, o)
            np.testing.assert_allclose(fm, -m * f, rtol=1e-12, atol=1e-13)
