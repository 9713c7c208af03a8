"""The product's TreeMesh containers (trixicuda/mesh.py, a tree walk) equal
the oracle's own (oracle/treemesh.py, a finest-level raster with a Morton
sort) array for array: element order, Jacobians, node coordinates,
interfaces, L2 mortars and boundaries -- for uniform meshes, the refined
quadrants / octants of the parity tests and the batched ensemble, the
reference's euler_blob_mortar boxes and non-periodic meshes.  The oracle
computes on its own containers, so a convention error in the product's mesh
code would show up here and in every parity test."""
import numpy as np
import pytest

import trixicuda as T
from oracle.oracle import Oracle, basis

FIELDS = ("inverse_jacobian", "node_coordinates", "interface_neighbor_ids", "interface_orientations",
          "mortar_neighbor_ids", "mortar_large_sides", "mortar_orientations", "boundary_neighbor_ids",
          "boundary_neighbor_sides", "boundary_orientations")


def _box(lo, hi):
    return dict(type="box", coordinates_min=lo, coordinates_max=hi)


MESHES = [
    ("1d-L4", (-1.0,), (1.0,), 4, [], True),
    ("2d-L3", (-2.0, -2.0), (2.0, 2.0), 3, [], True),
    ("2d-L7", (-2.0, -2.0), (2.0, 2.0), 7, [], True),
    ("3d-L3", (-2.0,) * 3, (2.0,) * 3, 3, [], True),
    ("2d-L3-quadrant", (-1.0, -1.0), (1.0, 1.0), 3, [_box((0.0, 0.0), (1.0, 1.0))], True),
    ("3d-L2-octant", (-1.0,) * 3, (1.0,) * 3, 2, [_box((0.0,) * 3, (1.0,) * 3)], True),
    ("2d-L6-quadrant", (-2.0, -2.0), (2.0, 2.0), 6, [_box((0.0, 0.0), (2.0, 2.0))], True),
    ("2d-mortar-strip", (-1.0, -1.0), (1.0, 1.0), 2, [_box((0.0, -1.0), (1.0, 1.0))], True),
    ("3d-two-boxes", (-1.0,) * 3, (1.0,) * 3, 2, [_box((0.0, -1.0, -1.0), (1.0, 1.0, 1.0)),
                                                  _box((0.0, -0.5, -0.5), (0.5, 0.5, 0.5))], True),
    ("2d-blob", (-32.0, -32.0), (32.0, 32.0), 4, [_box((-40.0, -5.0), (40.0, 5.0))] * 2, True),
    ("2d-nonperiodic", (0.0, 0.0), (2.0, 2.0), 3, [], False),
    ("2d-nonperiodic-quadrant", (0.0, 0.0), (2.0, 2.0), 3, [_box((0.0, 0.0), (1.0, 1.0))], False),
    ("3d-nonperiodic", (0.0,) * 3, (2.0,) * 3, 2, [], False),
    ("1d-nonperiodic", (0.0,), (2.0,), 3, [], False),
]


@pytest.mark.parametrize("name,lo,hi,level,patches,periodic", MESHES, ids=[m[0] for m in MESHES])
def test_oracle_containers_equal_product_containers(name, lo, hi, level, patches, periodic):
    d = len(lo)
    mesh = T.TreeMesh(lo if d > 1 else lo[0], hi if d > 1 else hi[0], initial_refinement_level=level,
                      refinement_patches=patches, periodicity=periodic)
    polydeg = 3
    mine = mesh.build_containers(T.LobattoLegendreBasisGPU(polydeg).nodes)
    theirs = Oracle.own_containers(mesh, polydeg)
    assert mine.nelements == theirs.nelements
    for f in FIELDS:
        a, b = np.asarray(getattr(mine, f)), np.asarray(getattr(theirs, f))
        assert a.shape == b.shape, (f, a.shape, b.shape)
        assert np.array_equal(a, b), f


def test_lgl_nodes_of_both_sides_agree():
    """The product's LGL nodes (libtrixi's host basis) and the oracle's are the
    same doubles, so node coordinates built from either agree bit for bit."""
    for p in range(1, 6):
        assert np.array_equal(T.LobattoLegendreBasisGPU(p).nodes, basis(p)["nodes"])


def test_oracle_workload_state_equals_product_state():
    """oracle/workloads.py restates the seeded 2D Euler initial condition of
    the benchmark; on the oracle's own mesh it gives the product's state bit
    for bit."""
    import bench
    from oracle.workloads import euler2d_fd_workload

    _, u, nel = euler2d_fd_workload(level=4, polydeg=3)
    mesh, eq, ic, solver = bench.build_problem("fp64")
    cont = T.TreeMesh((-2.0, -2.0), (2.0, 2.0), initial_refinement_level=4).build_containers(solver.basis.nodes)
    x = cont.node_coordinates.reshape(-1, 2).T
    assert nel == cont.nelements
    assert np.array_equal(u, ic(x, 0.0, eq).T.reshape(u.shape))


def test_cpu_baseline_leg_imports_no_product_code():
    """bench.py's CPU leg (cpu_baseline, the --impl reference arm) runs on
    oracle code alone: it imports no trixicuda module and maps no
    libtrixi_b200.so."""
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    code = ("import sys, bench\n"
            "r = bench.cpu_baseline(seconds_target=0.05, nthreads=2)\n"
            "assert r['value'] > 0\n"
            "bad = [m for m in sys.modules if m.split('.')[0] == 'trixicuda']\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert not bad, bad\n"
            "assert 'libtrixi_b200' not in maps\n"
            "print('ok')\n")
    res = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "ok" in res.stdout, res.stderr[-2000:]
