"""Multi-rank partitioning (CPU, gloo): element ranges of the Morton order
with a ghost layer refreshed by point-to-point halo exchange.  Every rank
evaluates the rhs of its local mesh (owned + ghosts) with the CPU oracle;
the owned parts, gathered, equal the single-rank rhs bit for bit, and so do
RK steps with one exchange per stage.  World sizes 2 and 3; a mortar mesh
and a 3D mesh are included."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem(kind):
    import trixicuda as T

    if kind == "euler2d":
        eq = T.CompressibleEulerEquations2D(1.4)
        solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_ranocha,
                            volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
        mesh = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=3,
                          refinement_patches=[dict(type="box", coordinates_min=(0.0, 0.0), coordinates_max=(2.0, 2.0))])
        ic = T.initial_condition_fourier_euler(eq, seed=5, kmax=3)
    else:
        eq = T.LinearScalarAdvectionEquation3D((0.2, -0.7, 0.5))
        solver = T.DGSEMGPU(polydeg=2, surface_flux=T.flux_lax_friedrichs)
        mesh = T.TreeMesh((-1.0,) * 3, (1.0,) * 3, initial_refinement_level=2)
        ic = T.initial_condition_convergence_test
    cont = mesh.build_containers(solver.basis.nodes)
    x = cont.node_coordinates.reshape(-1, mesh.ndims).T
    u = np.ascontiguousarray(ic(x, 0.0, eq).T.reshape((cont.nelements,) + (solver.polydeg + 1,) * mesh.ndims
                                                        + (eq.nvariables,)))
    return eq, solver, cont, u


def _oracle(eq, solver, cont):
    from oracle.oracle import Oracle

    class _S:
        pass

    s = _S()
    s.equations, s.solver, s.containers = eq, solver, cont
    return Oracle.from_semi(s)


def _worker(rank, world, port, kind, out_q):
    import sys

    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from trixicuda.partition import build_local, halo_exchange, partition_ranges
        from trixicuda.time_integration import CK2N54_A, CK2N54_B

        eq, solver, cont, u_glob = _problem(kind)
        ranges = partition_ranges(cont.nelements, world)
        part = build_local(cont, ranges, rank)
        ids = np.concatenate([part.owned, part.ghosts])
        u_loc = torch.from_numpy(u_glob[ids].copy())
        u_loc[part.nowned:] = 0.0
        halo_exchange(u_loc, part)
        # face-trace exchange: exactly the received nodes of the ghosts are
        # filled, with the owners' values, and every message is a face trace
        nv = u_glob.shape[-1]
        rows, ref_rows = u_loc.numpy().reshape(-1, nv), u_glob[ids].reshape(-1, nv)
        recv = np.concatenate([part.recv_nodes[r] for r in sorted(part.recv_nodes)])
        nn = int(np.prod(u_glob.shape[1:-1]))
        ghosts_ok = bool(np.array_equal(rows[recv], ref_rows[recv]) and np.all(recv >= part.nowned * nn)
                         and sum(len(v) for v in part.send_nodes.values())
                         < nn * sum(len(v) for v in part.send.values()))
        orc = _oracle(eq, solver, part.containers)
        du = orc.rhs(u_loc.numpy())[: part.nowned]
        # two RK steps, one halo exchange per stage
        dt = 1e-3
        u = u_loc.clone()
        k = torch.zeros_like(u)
        for _ in range(2):
            for a, b in zip(CK2N54_A, CK2N54_B):
                halo_exchange(u, part)
                d = torch.from_numpy(orc.rhs(u.numpy()))
                k = a * k + dt * d
                u = u + b * k
        out_q.put((rank, part.owned, du, u.numpy()[: part.nowned], ghosts_ok, {r: len(v) for r, v in part.send.items()}))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("kind,world", [("euler2d", 2), ("euler2d", 3), ("adv3d", 2)])
def test_partitioned_rhs_and_rk_equal_single_rank(kind, world):
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, kind, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    eq, solver, cont, u = _problem(kind)
    orc = _oracle(eq, solver, cont)
    du_ref = orc.rhs(u)
    u_ref, _ = orc.rk_ck2n54(u, 0.0, 1e-3, 2)
    covered = np.zeros(cont.nelements, dtype=bool)
    for rank, owned, du, uu, ghosts_ok, sends in sorted(results, key=lambda r: r[0]):
        assert ghosts_ok
        assert sends, "every rank exchanges with a neighbour"
        assert np.array_equal(du, du_ref[owned])
        np.testing.assert_allclose(uu, u_ref[owned], rtol=0, atol=1e-14)
        covered[owned] = True
    assert covered.all()


def test_partition_ranges_balanced():
    from trixicuda.partition import partition_ranges

    r = partition_ranges(1000, 7)
    sizes = [b - a for a, b in r]
    assert r[0][0] == 0 and r[-1][1] == 1000 and max(sizes) - min(sizes) <= 1
