"""Non-periodic TreeMeshes, Dirichlet boundaries and source terms: the mesh's
boundaries container and the oracle, without a GPU.  Mirrors the reference's
non-periodic set-ups (test/tree_dgsem_2d/euler_source_terms_nonperiodic.jl:
BoundaryConditionDirichlet(initial_condition_convergence_test) on every side,
source_terms_convergence_test)."""
import ctypes as C

import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import Oracle


def _euler(d):
    return {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
            3: T.CompressibleEulerEquations3D}[d](1.4)


@pytest.mark.parametrize("d,level,refined", [(1, 3, False), (2, 2, False), (2, 3, True), (3, 2, False), (3, 2, True)])
def test_nonperiodic_faces_covered_once(d, level, refined):
    patches = [dict(type="box", coordinates_min=(0.0,) * d, coordinates_max=(1.0,) * d)] if refined and d > 1 else []
    mesh = T.TreeMesh((0.0,) * d, (2.0,) * d, initial_refinement_level=level, refinement_patches=patches,
                      periodicity=False)
    cont = mesh.build_containers(np.array([-1.0, 0.0, 1.0]))
    count = np.zeros((cont.nelements, 2 * d), dtype=int)
    for (l, r), o in zip(cont.interface_neighbor_ids, cont.interface_orientations):
        count[l - 1, 2 * (o - 1) + 1] += 1
        count[r - 1, 2 * (o - 1)] += 1
    nc = 2 ** (d - 1)
    for ids, ls, o in zip(cont.mortar_neighbor_ids, cont.mortar_large_sides, cont.mortar_orientations):
        for s in ids[:nc]:
            count[s - 1, 2 * (o - 1) + (ls - 1)] += 1
        count[ids[nc] - 1, 2 * (o - 1) + (1 if ls == 1 else 0)] += 1
    for e, side, o in zip(cont.boundary_neighbor_ids, cont.boundary_neighbor_sides, cont.boundary_orientations):
        count[e - 1, 2 * (o - 1) + (1 if side == 1 else 0)] += 1
    assert np.all(count == 1)
    # boundaries ordered by direction (x_neg, x_pos, ...), sides 2 on lower faces
    dirs = 2 * (cont.boundary_orientations - 1) + (cont.boundary_neighbor_sides == 1)
    assert np.all(np.diff(dirs) >= 0)
    assert list(np.bincount(dirs, minlength=2 * d)) == list(cont.n_boundaries_per_direction)
    # the boundary nodes lie on the domain boundary
    N = 3
    for e, side, o in zip(cont.boundary_neighbor_ids, cont.boundary_neighbor_sides, cont.boundary_orientations):
        xs = cont.node_coordinates[e - 1].reshape(-1, d)[:, o - 1]
        assert np.isclose(xs.max() if side == 1 else xs.min(), 2.0 if side == 1 else 0.0)


def test_periodic_mesh_has_no_boundaries():
    mesh = T.TreeMesh((0.0, 0.0), (2.0, 2.0), initial_refinement_level=2)
    cont = mesh.build_containers(np.array([-1.0, 1.0]))
    assert cont.nboundaries == 0 and cont.ninterfaces == 2 * 16


def _oracle(d, level, polydeg=3, bc=1, bc_params=(2.0, 0.1, 2.0), source=1, vol=0, vflux=2, sflux=0):
    eq = _euler(d)
    mesh = T.TreeMesh((0.0,) * d, (2.0,) * d, initial_refinement_level=level, periodicity=False)
    solver = T.DGSEMGPU(polydeg=polydeg)
    cont = mesh.build_containers(solver.basis.nodes)
    orc = Oracle(cont, d, polydeg, eq.nvariables, eq.code, gamma=1.4, volume_integral=vol, volume_flux=vflux,
                 surface_flux=sflux, boundary_function=bc, boundary_params=bc_params, source_terms=source)
    return eq, cont, orc


@pytest.mark.parametrize("d", [1, 2, 3])
def test_oracle_source_matches_host_formula(d):
    eq, cont, orc = _oracle(d, 1)
    du = np.zeros(orc.lib.oracle_size(orc._h, 0))
    orc.sources(du, 0.37)
    x = cont.node_coordinates.reshape(-1, d).T
    ref = T.source_terms_convergence_test(None, x, 0.37, eq).T.reshape(-1)
    np.testing.assert_allclose(du, ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("d,vol", [(1, 0), (2, 0), (2, 1), (3, 1)])
def test_free_stream_with_constant_dirichlet_boundaries(d, vol):
    eq = _euler(d)
    state = np.concatenate([[1.2], 1.2 * np.array([0.3, -0.2, 0.1][:d]), [2.0 / 0.4 + 0.5 * 1.2 * 0.14]])
    _, cont, orc = _oracle(d, 2, bc=0, bc_params=state, source=0, vol=vol, vflux=1, sflux=0)
    u = np.broadcast_to(state, (cont.nelements,) + (4,) * d + (eq.nvariables,)).copy()
    du = orc.rhs(u, 0.0)
    assert np.max(np.abs(du)) < 1e-12


def _eoc_error(d, level, p=3, t_end=0.1):
    eq, cont, orc = _oracle(d, level, polydeg=p)
    x = cont.node_coordinates.reshape(-1, d).T
    shape = (cont.nelements,) + (p + 1,) * d + (eq.nvariables,)
    u = np.ascontiguousarray(T.initial_condition_convergence_test(x, 0.0, eq).T.reshape(shape))
    k = np.zeros_like(u)
    h = 2.0 / 2 ** level
    nsteps = int(np.ceil(t_end / (0.4 * h / (p + 1) / 3.0)))
    dt = t_end / nsteps
    pd = C.POINTER(C.c_double)
    orc.lib.oracle_rk_ck2n54(orc._h, u.ctypes.data_as(pd), k.ctypes.data_as(pd), 0.0, dt, nsteps)
    ue = T.initial_condition_convergence_test(x, t_end, eq).T.reshape(shape)
    return float(np.sqrt(np.mean((u - ue) ** 2)))


@pytest.mark.parametrize("d,levels,min_eoc", [(1, (3, 4), 3.7), (2, (2, 3), 3.3)])
def test_convergence_with_dirichlet_boundaries_and_sources(d, levels, min_eoc):
    """The manufactured solution converges at order ~polydeg+1 with its
    source term and exact Dirichlet boundary states (time-dependent: the
    boundary states follow the RK stage times t + c_s dt)."""
    e0, e1 = (_eoc_error(d, lv) for lv in levels)
    assert np.log2(e0 / e1) > min_eoc, (e0, e1)


@pytest.mark.parametrize("d,sflux", [(1, 7), (2, 7), (3, 6)])
def test_free_stream_with_dirichlet_boundaries_hll_family(d, sflux):
    """flux_hlle / flux_hll at Dirichlet faces holding the free stream: the
    HLL fluxes are consistent, so the constant state stays put."""
    eq = _euler(d)
    state = np.concatenate([[1.2], 1.2 * np.array([0.3, -0.2, 0.1][:d]), [2.0 / 0.4 + 0.5 * 1.2 * 0.14]])
    _, cont, orc = _oracle(d, 2, bc=0, bc_params=state, source=0, vol=1, vflux=1, sflux=sflux)
    u = np.broadcast_to(state, (cont.nelements,) + (4,) * d + (eq.nvariables,)).copy()
    assert np.max(np.abs(orc.rhs(u, 0.0))) < 1e-12
