"""The reference's 3D Euler convergence set-up (test/tree_dgsem_3d/
euler_convergence.jl:9-26): initial_condition_eoc_test_coupled_euler_gravity
with source_terms_eoc_test_euler, gamma = 2, flux_hll surface flux, weak form,
periodic [0, 2]^3.  Both functions are restated from the published
manufactured solution of the Euler-gravity test (Schlottke-Lakemper et al.,
JCP 442 (2021)); these CPU pins check the restatements against each other
(device formula via the host copy, oracle by the chain rule) and the
convergence order the source must produce."""
import ctypes as C

import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import FLUX_HLL, VOL_WEAK, Oracle


def _setup(d, level, p=3):
    eq = {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
          3: T.CompressibleEulerEquations3D}[d](2.0)
    mesh = T.TreeMesh((0.0,) * d if d > 1 else 0.0, (2.0,) * d if d > 1 else 2.0, initial_refinement_level=level)
    cont = Oracle.own_containers(mesh, p)
    orc = Oracle(cont, d, p, eq.nvariables, eq.code, gamma=2.0, volume_integral=VOL_WEAK, surface_flux=FLUX_HLL,
                 source_terms=T._lib.SOURCE_EOC_TEST_EULER)
    return eq, cont, orc


@pytest.mark.parametrize("d", [1, 2, 3])
def test_source_host_formula_equals_oracle_chain_rule(d):
    eq, cont, orc = _setup(d, 1)
    du = np.zeros(orc.lib.oracle_size(orc._h, 0))
    orc.sources(du, 0.37)
    x = cont.node_coordinates.reshape(-1, d).T
    ref = T.source_terms_eoc_test_euler(None, x, 0.37, eq).T.reshape(-1)
    np.testing.assert_allclose(du, ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_source_is_the_residual_of_the_manufactured_solution(d):
    """S = du/dt + div F(u) at random points, with the derivatives of the
    initial condition taken by central differences (h = 1e-5)."""
    eq = {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
          3: T.CompressibleEulerEquations3D}[d](2.0)
    ic = T.initial_condition_eoc_test_coupled_euler_gravity
    rng = np.random.default_rng(3)
    x = rng.uniform(0.0, 2.0, (d, 16))
    t, h = 0.3, 1e-5

    def flux(u, k):
        rho = u[0]
        v = u[1:1 + d] / rho
        p = (eq.gamma - 1) * (u[-1] - 0.5 * rho * np.sum(v * v, axis=0))
        f = np.empty_like(u)
        f[0] = u[1 + k]
        f[1:1 + d] = u[1 + k] * v
        f[1 + k] += p
        f[-1] = (u[-1] + p) * v[k]
        return f

    res = (ic(x, t + h, eq) - ic(x, t - h, eq)) / (2 * h)
    for k in range(d):
        e = np.zeros((d, 1))
        e[k] = h
        res += (flux(ic(x + e, t, eq), k) - flux(ic(x - e, t, eq), k)) / (2 * h)
    np.testing.assert_allclose(T.source_terms_eoc_test_euler(None, x, t, eq), res, rtol=1e-8, atol=1e-8)


def _error(d, level, p=3, t_end=0.2):
    eq, cont, orc = _setup(d, level, p)
    ic = T.initial_condition_eoc_test_coupled_euler_gravity
    x = cont.node_coordinates.reshape(-1, d).T
    shape = (cont.nelements,) + (p + 1,) * d + (eq.nvariables,)
    u = np.ascontiguousarray(ic(x, 0.0, eq).T.reshape(shape))
    k = np.zeros_like(u)
    hcell = 2.0 / 2 ** level
    nsteps = int(np.ceil(t_end / (0.3 * hcell / (p + 1) / (1.0 + 1.2))))
    dt = t_end / nsteps
    pd = C.POINTER(C.c_double)
    orc.lib.oracle_rk_ck2n54(orc._h, u.ctypes.data_as(pd), k.ctypes.data_as(pd), 0.0, dt, nsteps)
    ue = ic(x, t_end, eq).T.reshape(shape)
    return float(np.sqrt(np.mean((u - ue) ** 2)))


@pytest.mark.parametrize("d,levels,min_eoc", [(1, (3, 4), 3.5), (2, (2, 3), 3.3), (3, (1, 2), 3.0)])
def test_convergence_order(d, levels, min_eoc):
    e0, e1 = (_error(d, lv) for lv in levels)
    assert np.log2(e0 / e1) > min_eoc, (e0, e1, np.log2(e0 / e1))
