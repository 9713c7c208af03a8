"""Ghost elements in libtrixi_b200 (the local mesh of a partitioned run):
with the ghost layer filled from the global state, the owned part of the
local rhs equals the global rhs bit for bit (one GPU, no exchange)."""
import numpy as np
import pytest

import trixicuda as T
from trixicuda.partition import build_local, partition_ranges

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nranks,refined", [(2, False), (3, True)])
def test_local_mesh_with_ghosts_matches_global(nranks, refined, cuda):
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_ranocha,
                        volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    patches = [dict(type="box", coordinates_min=(0.0, 0.0), coordinates_max=(2.0, 2.0))] if refined else []
    mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=4, refinement_patches=patches)
    ic = T.initial_condition_fourier_euler(eq, seed=9, kmax=4)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver)
    u = semi.compute_coefficients()
    du = cuda.empty_like(u)
    T.rhs_gpu(du, u, semi, 0.0)
    ranges = partition_ranges(semi.nelements, nranks)
    for r in range(nranks):
        part = build_local(semi.containers, ranges, r)
        local = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, containers=part.containers)
        ids = cuda.as_tensor(np.concatenate([part.owned, part.ghosts]), device=u.device)
        ul = u[ids].contiguous()
        dul = cuda.empty_like(ul)
        T.rhs_gpu(dul, ul, local, 0.0)
        T.synchronize(local)
        assert cuda.equal(dul[: part.nowned], du[cuda.as_tensor(part.owned, device=u.device)])


@pytest.mark.parametrize("kind,nranks", [("euler_fd", 2), ("euler_fd", 3), ("adv_weak", 2), ("euler_sc", 2)])
def test_partitioned_rk_steps_colocated_match_single_domain(kind, nranks, cuda):
    """PartitionedSemidiscretizationGPU on one GPU: nranks partitions in one
    process, their ghost traces refreshed by device copies before every stage
    (rk_steps_colocated, the same packed plan the NCCL messages carry).  Two
    CarpenterKennedy2N54 steps give the owned elements the single-domain
    result bit for bit.  Face traces for flux differencing and the weak form,
    whole ghost elements for shock capturing."""
    from trixicuda.partition import PartitionedSemidiscretizationGPU, rk_steps_colocated
    from problems import make

    d = 3 if kind == "adv_weak" else 2
    mesh, eq, ic, solver, _ = make(kind, d, 2 if d == 3 else 3, refined=(kind != "euler_sc"))
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver)
    u = semi.compute_coefficients()
    dt = 0.2 / float(np.max(semi.containers.inverse_jacobian)) / 4
    uref, kref = u.clone(), cuda.zeros_like(u)
    T.rk_steps(uref, kref, 0.0, dt, 2, semi)
    ranks = [PartitionedSemidiscretizationGPU(mesh, eq, ic, solver, r, nranks) for r in range(nranks)]
    assert ranks[0].part.mode == ("elements" if kind == "euler_sc" else "faces")
    us = [rk.local_state(u) for rk in ranks]
    if kind != "euler_sc":  # face traces: the ghosts start empty, only the exchange fills them
        for rk, ul in zip(ranks, us):
            ul[rk.part.nowned:] = 0.0
    ks = [cuda.zeros_like(ul) for ul in us]
    rk_steps_colocated(ranks, us, ks, 0.0, dt, 2)
    cuda.cuda.synchronize()
    for rk, ul in zip(ranks, us):
        owned = cuda.as_tensor(rk.part.owned, device=u.device)
        assert cuda.equal(ul[: rk.part.nowned], uref[owned])


def test_partition_refuses_boundaries_and_sources(cuda):
    from trixicuda.partition import PartitionedSemidiscretizationGPU

    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs)
    mesh = T.TreeMesh((0.0, 0.0), (2.0, 2.0), initial_refinement_level=2, periodicity=False)
    with pytest.raises(NotImplementedError):
        PartitionedSemidiscretizationGPU(mesh, eq, T.initial_condition_convergence_test, solver, 0, 2,
                                         boundary_conditions=T.BoundaryConditionDirichlet(
                                             T.initial_condition_convergence_test))
    mesh = T.TreeMesh((0.0, 0.0), (2.0, 2.0), initial_refinement_level=2)
    with pytest.raises(NotImplementedError):
        PartitionedSemidiscretizationGPU(mesh, eq, T.initial_condition_convergence_test, solver, 0, 2,
                                         source_terms=T.source_terms_convergence_test)
