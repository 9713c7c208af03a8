"""Element partitioning and ghost-layer halo exchange for several GPUs.

The reference is single-GPU.  A TreeMesh partitions naturally into
contiguous element ranges of its depth-first Morton order; every rank then
needs, before each rhs evaluation, the states of the elements across its
partition boundary (the "ghost layer": elements sharing an interface or a
mortar with an owned element).  This module builds, per rank,

* the local mesh: owned elements first, ghosts last, with the interfaces and
  mortars that touch an owned element (ghost faces facing outside the local
  set stay open -- libtrixi_b200 accepts that for the trailing
  `nghost_elements`, whose rhs is discarded);
* the exchange plan: which owned elements each neighbour rank needs, and
  which ghost slots receive from each rank;

and exchanges the ghost states with point-to-point torch.distributed
messages (NCCL between GPUs, gloo on CPU).  There is no collective on the data
path; a time step only needs a global reduction for max_dt.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import Containers


def partition_ranges(nelements: int, nranks: int):
    """Balanced contiguous ranges [start, stop) of the element order."""
    bounds = [round(r * nelements / nranks) for r in range(nranks + 1)]
    return [(bounds[r], bounds[r + 1]) for r in range(nranks)]


def owner_of(ranges):
    stops = np.array([b for _, b in ranges])

    def f(e):
        return int(np.searchsorted(stops, e, side="right"))

    return f


@dataclass
class LocalPartition:
    rank: int
    nranks: int
    owned: np.ndarray                 # global ids (0-based) of owned elements, in order
    ghosts: np.ndarray                # global ids of ghosts, in order
    containers: Containers            # local mesh (owned then ghosts), nghost_elements set
    send: dict = field(default_factory=dict)   # rank -> local ids (owned) to send
    recv: dict = field(default_factory=dict)   # rank -> local ids (ghost slots) to fill

    @property
    def nowned(self) -> int:
        return int(self.owned.size)


def build_local(cont: Containers, ranges, rank: int) -> LocalPartition:
    start, stop = ranges[rank]
    owner = owner_of(ranges)
    owned = np.arange(start, stop, dtype=np.int64)
    own_set = set(owned.tolist())
    d = cont.ndims
    nc = 2 ** (d - 1)
    # interfaces and mortars touching an owned element (global, 0-based)
    ifs = [(k, int(l) - 1, int(r) - 1) for k, (l, r) in enumerate(cont.interface_neighbor_ids)
           if (l - 1) in own_set or (r - 1) in own_set]
    mos = [m for m in range(cont.nmortars) if any((int(x) - 1) in own_set for x in cont.mortar_neighbor_ids[m])]
    ghost_set = set()
    for _, l, r in ifs:
        for e in (l, r):
            if e not in own_set:
                ghost_set.add(e)
    for m in mos:
        for x in cont.mortar_neighbor_ids[m]:
            if (int(x) - 1) not in own_set:
                ghost_set.add(int(x) - 1)
    ghosts = np.array(sorted(ghost_set), dtype=np.int64)
    local_ids = np.concatenate([owned, ghosts])
    g2l = {int(g): i for i, g in enumerate(local_ids)}
    if_nid = np.array([[g2l[l] + 1, g2l[r] + 1] for _, l, r in ifs], dtype=np.int64).reshape(-1, 2)
    if_ori = np.array([cont.interface_orientations[k] for k, _, _ in ifs], dtype=np.int64)
    mo_nid = np.array([[g2l[int(x) - 1] + 1 for x in cont.mortar_neighbor_ids[m]] for m in mos],
                      dtype=np.int64).reshape(-1, nc + 1)
    local = Containers(
        ndims=d, nnodes=cont.nnodes, nelements=int(local_ids.size),
        inverse_jacobian=cont.inverse_jacobian[local_ids].copy(),
        node_coordinates=cont.node_coordinates[local_ids].copy(),
        element_level=cont.element_level[local_ids].copy(),
        interface_neighbor_ids=if_nid, interface_orientations=if_ori,
        mortar_neighbor_ids=mo_nid,
        mortar_large_sides=np.array([cont.mortar_large_sides[m] for m in mos], dtype=np.int64),
        mortar_orientations=np.array([cont.mortar_orientations[m] for m in mos], dtype=np.int64),
    )
    local.nghost_elements = int(ghosts.size)
    part = LocalPartition(rank, len(ranges), owned, ghosts, local)
    for i, g in enumerate(ghosts):
        part.recv.setdefault(owner(int(g)), []).append(owned.size + i)
    # what the other ranks need from us: our elements that are their ghosts
    for r in range(len(ranges)):
        if r == rank:
            continue
        theirs = _ghost_ids(cont, ranges, r)
        mine = [int(g) - start for g in theirs if start <= g < stop]
        if mine:
            part.send[r] = mine
    part.send = {r: np.array(v, dtype=np.int64) for r, v in part.send.items()}
    part.recv = {r: np.array(v, dtype=np.int64) for r, v in part.recv.items()}
    return part


def _ghost_ids(cont: Containers, ranges, rank: int) -> np.ndarray:
    start, stop = ranges[rank]

    def owned(e):
        return start <= e < stop

    gs = set()
    for l, r in cont.interface_neighbor_ids:
        l, r = int(l) - 1, int(r) - 1
        if owned(l) and not owned(r):
            gs.add(r)
        if owned(r) and not owned(l):
            gs.add(l)
    for ids in cont.mortar_neighbor_ids:
        ids = [int(x) - 1 for x in ids]
        if any(owned(x) for x in ids):
            gs.update(x for x in ids if not owned(x))
    return np.array(sorted(gs), dtype=np.int64)


def halo_exchange(u_local, part: LocalPartition, group=None):
    """Fill the ghost elements of u_local (shape (nlocal, ...)) from their owners."""
    import torch
    import torch.distributed as dist

    ops, bufs = [], []
    for r, ids in sorted(part.send.items()):
        buf = u_local[torch.as_tensor(ids, device=u_local.device)].contiguous()
        bufs.append(buf)
        ops.append(dist.P2POp(dist.isend, buf, r, group))
    recv_bufs = {}
    for r, ids in sorted(part.recv.items()):
        buf = torch.empty((len(ids),) + tuple(u_local.shape[1:]), dtype=u_local.dtype, device=u_local.device)
        recv_bufs[r] = buf
        ops.append(dist.P2POp(dist.irecv, buf, r, group))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    for r, buf in recv_bufs.items():
        u_local[torch.as_tensor(part.recv[r], device=u_local.device)] = buf
    return u_local


class PartitionedSemidiscretizationGPU:
    """One rank's share of a partitioned problem on its GPU: the library
    handle of the local mesh (owned + ghosts) and the exchange plan.  Each RK
    stage refreshes the ghosts (NCCL point-to-point) and runs the fused stage
    kernel on the local arrays; ghost results are discarded."""

    def __init__(self, mesh, equations, initial_condition, solver, rank, nranks, precision="fp64", device=None):
        from .semidiscretization import SemidiscretizationHyperbolicGPU

        self.global_containers = mesh.build_containers(solver.basis.nodes)
        self.ranges = partition_ranges(self.global_containers.nelements, nranks)
        self.part = build_local(self.global_containers, self.ranges, rank)
        self.semi = SemidiscretizationHyperbolicGPU(mesh, equations, initial_condition, solver,
                                                    precision=precision, device=device,
                                                    containers=self.part.containers)

    def rk_steps(self, u_local, k_local, dt, nsteps, group=None):
        import torch

        from .semidiscretization import rk_stage
        from .time_integration import CK2N54_A, CK2N54_B

        other = torch.empty_like(u_local)
        cur, nxt = u_local, other
        for _ in range(nsteps):
            for a, b in zip(CK2N54_A, CK2N54_B):
                halo_exchange(cur.view(self.semi.u_shape()), self.part, group)
                rk_stage(nxt, cur, k_local, a, b, dt, 0.0, self.semi)
                cur, nxt = nxt, cur
        if cur is not u_local:
            u_local.copy_(cur)
        return u_local
