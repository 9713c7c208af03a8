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
