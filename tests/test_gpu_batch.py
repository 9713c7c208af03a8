"""Batched ensembles: a heterogeneous batch (mixed ndims, polydeg,
equations, mortar meshes) advanced through trixi_batch_* must give, per
instance, exactly what the single-problem path gives, and match the oracle."""
import numpy as np
import pytest

import trixicuda as T
from conftest import assert_rel
from trixicuda.batch import BatchedSemidiscretizationGPU, Problem

pytestmark = pytest.mark.gpu


def _problems():
    probs = []
    specs = [("adv", 2, 2, 2, False), ("euler", 2, 2, 3, True), ("adv", 3, 1, 4, True), ("euler", 2, 3, 2, False),
             ("adv", 2, 3, 3, True), ("adv", 3, 2, 2, False), ("euler", 2, 2, 3, False), ("adv", 2, 2, 2, False)]
    for i, (fam, d, lvl, p, ref) in enumerate(specs):
        lo, hi = (-2.0, 2.0) if fam == "euler" else (-1.0, 1.0)
        patches = [dict(type="box", coordinates_min=(0.0,) * d, coordinates_max=(hi,) * d)] if ref else []
        mesh = T.TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=lvl, refinement_patches=patches)
        if fam == "euler":
            eq = T.CompressibleEulerEquations2D(1.4)
            solver = T.DGSEMGPU(polydeg=p, surface_flux=T.flux_ranocha,
                                volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
            ic = T.initial_condition_fourier_euler(eq, seed=100 + i, kmax=3, xmin=lo, xmax=hi)
        else:
            eq = (T.LinearScalarAdvectionEquation2D((0.2, -0.7)) if d == 2
                  else T.LinearScalarAdvectionEquation3D((0.2, -0.7, 0.5)))
            solver = T.DGSEMGPU(polydeg=p, surface_flux=T.flux_lax_friedrichs)
            ic = T.initial_condition_fourier_advection(eq, seed=100 + i, kmax=3, xmin=lo, xmax=hi)
        probs.append(Problem(mesh, eq, ic, solver))
    return probs


def _host_ic(pb, cont):
    x = cont.node_coordinates.reshape(-1, pb.mesh.ndims).T
    return pb.initial_condition(x, 0.0, pb.equations).T


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_single_problems(precision, cuda):
    probs = _problems()
    batch = BatchedSemidiscretizationGPU(probs, precision=precision)
    assert batch.ngroups < len(probs)  # instances of a kind share a group
    u = cuda.empty(batch.total_values, dtype=cuda.float64, device=batch.device)
    for i, pb in enumerate(probs):
        batch.view(u, i).copy_(cuda.from_numpy(np.ascontiguousarray(_host_ic(pb, batch.containers[i]))
                                               .reshape(batch.shape(i))))
    du = cuda.empty_like(u)
    batch.rhs(du, u)
    dts = batch.stable_dt(u)
    ug, kg = u.clone(), cuda.zeros_like(u)
    batch.rk_steps(ug, kg, dts, 3, use_graph=True)
    un, kn = u.clone(), cuda.zeros_like(u)
    batch.rk_steps(un, kn, dts, 3, use_graph=False)
    cuda.cuda.synchronize()
    assert cuda.equal(ug, un) and cuda.equal(kg, kn)  # graph replay == direct launches
    # the branch tuner ran at the graph build, on copies of the state
    branches, timings = batch.tuning()
    assert branches in timings and all(ms > 0 for ms in timings.values())
    assert 1 in timings and max(timings) <= batch.ngroups
    for i, pb in enumerate(probs):
        semi = T.SemidiscretizationHyperbolicGPU(pb.mesh, pb.equations, pb.initial_condition, pb.solver,
                                                 precision=precision)
        ui = batch.view(u, i).contiguous()
        dui = cuda.empty_like(ui)
        T.rhs_gpu(dui, ui, semi, 0.0)
        uu, kk = ui.clone(), cuda.zeros_like(ui)
        T.rk_steps(uu, kk, 0.0, float(dts[i]), 3, semi)
        cuda.cuda.synchronize()
        assert cuda.equal(batch.view(du, i), dui), i
        assert cuda.equal(batch.view(ug, i), uu), i


def test_batch_matches_oracle(cuda):
    from oracle.oracle import Oracle

    probs = _problems()
    batch = BatchedSemidiscretizationGPU(probs, precision="fp64")
    u = cuda.empty(batch.total_values, dtype=cuda.float64, device=batch.device)
    hosts = []
    for i, pb in enumerate(probs):
        h = np.ascontiguousarray(_host_ic(pb, batch.containers[i])).reshape(batch.shape(i))
        hosts.append(h)
        batch.view(u, i).copy_(cuda.from_numpy(h))
    du = cuda.empty_like(u)
    batch.rhs(du, u)
    cuda.cuda.synchronize()
    for i, pb in enumerate(probs):

        class _S:
            pass

        s = _S()
        s.equations, s.solver, s.containers, s.mesh = pb.equations, pb.solver, batch.containers[i], pb.mesh
        ref = Oracle.from_semi(s).rhs(hosts[i])
        assert_rel(batch.view(du, i).cpu().numpy(), ref, 1e-12, f"instance {i}")
