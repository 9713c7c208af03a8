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
* the exchange plan.  Face traces (the default): for every cut face, the
  nv N^(d-1) values of the trace of its owned side, which is all the local
  rhs reads of a ghost (interface fluxes and mortar projections take the
  neighbour's face nodes only); the plan lists (element, face) pairs in one
  order that both ranks derive from the global connectivity, so the sender
  packs and the receiver unpacks the same sequence.  Whole ghost elements for
  shock capturing, whose indicator smoothing needs every node of the ghost;

and exchanges them with point-to-point torch.distributed messages (NCCL
between GPUs, gloo on CPU), or with device copies between partitions held in
one process (rk_steps_colocated).  There is no collective on the data path; a
time step only needs a global reduction for max_dt.  The index tensors of a
plan are built once per device.
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
    # face-trace plan: rank -> local node ids (element * N^d + node) to send / fill
    send_nodes: dict = field(default_factory=dict)
    recv_nodes: dict = field(default_factory=dict)
    mode: str = "faces"               # "faces" or "elements"
    _dev: dict = field(default_factory=dict)   # device -> {(kind, rank): index tensor}

    @property
    def nowned(self) -> int:
        return int(self.owned.size)

    def index(self, kind, rank, device):
        """The plan's index tensor (kind 'send' / 'recv') for `rank` on `device`,
        built on the first call."""
        import torch

        key = (kind, rank)
        cache = self._dev.setdefault(str(device), {})
        if key not in cache:
            if self.mode == "faces":
                src = (self.send_nodes if kind == "send" else self.recv_nodes)[rank]
            else:
                src = (self.send if kind == "send" else self.recv)[rank]
            cache[key] = torch.as_tensor(np.asarray(src, dtype=np.int64), device=device)
        return cache[key]

    def peers(self, kind):
        table = (self.send_nodes if kind == "send" else self.recv_nodes) if self.mode == "faces" else \
            (self.send if kind == "send" else self.recv)
        return sorted(table)


def face_nodes(ndims: int, N: int, dim: int, upper: bool) -> np.ndarray:
    """Node indices (memory order, x fastest) of an element's face (dim, side),
    in the order of the face's remaining coordinates."""
    idx = np.arange(N ** ndims).reshape((N,) * ndims)  # idx[z, y, x] in memory order
    sl = [slice(None)] * ndims
    sl[ndims - 1 - dim] = N - 1 if upper else 0
    return idx[tuple(sl)].reshape(-1)


def _trace_plan(cont: Containers, ranges, src: int, dst: int):
    """(global element, dim, upper) of the faces whose traces rank src sends to
    rank dst, in the order of the global interfaces and then the global
    mortars (large element first, then the small ones): the traces of src's
    elements across an interface from a dst element, and, on every mortar
    that holds an element of dst, the mortar-face traces of its src
    elements."""
    s0, s1 = ranges[src]
    d0, d1 = ranges[dst]
    nc = 2 ** (cont.ndims - 1)
    out = []
    for (l, r), o in zip(cont.interface_neighbor_ids, cont.interface_orientations):
        l, r, dim = int(l) - 1, int(r) - 1, int(o) - 1
        if s0 <= l < s1 and d0 <= r < d1:
            out.append((l, dim, True))      # the left element's upper face
        if s0 <= r < s1 and d0 <= l < d1:
            out.append((r, dim, False))
    for m in range(cont.nmortars):
        ids = [int(x) - 1 for x in cont.mortar_neighbor_ids[m]]
        if not any(d0 <= x < d1 for x in ids):
            continue
        dim = int(cont.mortar_orientations[m]) - 1
        large_left = int(cont.mortar_large_sides[m]) == 1
        large, smalls = ids[nc], ids[:nc]
        if s0 <= large < s1:
            out.append((large, dim, large_left))
        for x in smalls:
            if s0 <= x < s1:
                out.append((x, dim, not large_left))
    return out


def build_local(cont: Containers, ranges, rank: int, mode: str = "faces") -> LocalPartition:
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
    part.mode = mode
    if mode == "faces":
        NN = cont.nnodes ** d
        fn = {(dim, up): face_nodes(d, cont.nnodes, dim, up) for dim in range(d) for up in (False, True)}
        for r in range(len(ranges)):
            if r == rank:
                continue
            out = _trace_plan(cont, ranges, rank, r)
            if out:
                part.send_nodes[r] = np.concatenate([(int(g) - start) * NN + fn[(dim, up)] for g, dim, up in out])
            inn = _trace_plan(cont, ranges, r, rank)
            if inn:
                part.recv_nodes[r] = np.concatenate([g2l[int(g)] * NN + fn[(dim, up)] for g, dim, up in inn])
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


def _rows(u_local, part: LocalPartition):
    """u_local viewed as the rows the plan indexes: nodes (nvars values each)
    for face traces, elements for whole ghosts."""
    n = u_local.shape[0]
    if part.mode == "faces":
        nv = u_local.shape[-1]
        return u_local.reshape(-1, nv)
    return u_local.reshape(n, -1)


def halo_exchange(u_local, part: LocalPartition, group=None):
    """Fill the ghost data of u_local (shape (nlocal, N.., nvars)) from their
    owners: point-to-point sends of the packed face traces (or whole
    elements), one message per neighbour rank and direction."""
    import torch.distributed as dist

    rows = _rows(u_local, part)
    ops, recv_bufs = [], {}
    for r in part.peers("send"):
        buf = rows.index_select(0, part.index("send", r, u_local.device))
        ops.append(dist.P2POp(dist.isend, buf, r, group))
    for r in part.peers("recv"):
        idx = part.index("recv", r, u_local.device)
        buf = rows.new_empty((idx.numel(), rows.shape[1]))
        recv_bufs[r] = buf
        ops.append(dist.P2POp(dist.irecv, buf, r, group))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    for r, buf in recv_bufs.items():
        rows.index_copy_(0, part.index("recv", r, u_local.device), buf)
    return u_local


def colocated_exchange(u_locals, parts):
    """halo_exchange for partitions held in one process (one device or
    several visible to it): the traces go by device copies, in the same
    packed order as the messages."""
    rows = [_rows(u, p) for u, p in zip(u_locals, parts)]
    for a, pa in enumerate(parts):
        for b in pa.peers("send"):
            src = rows[a].index_select(0, pa.index("send", b, u_locals[a].device)).to(u_locals[b].device)
            rows[b].index_copy_(0, parts[b].index("recv", a, u_locals[b].device), src)


class PartitionedSemidiscretizationGPU:
    """One rank's share of a partitioned problem on its GPU: the library
    handle of the local mesh (owned + ghosts) and the exchange plan.  Each RK
    stage refreshes the ghost traces (NCCL point-to-point) and runs the fused
    stage kernel on the local arrays; ghost results are discarded.  Periodic
    meshes without source terms only: the local meshes carry no boundaries
    container and the stages no source evaluation."""

    def __init__(self, mesh, equations, initial_condition, solver, rank, nranks, precision="fp64", device=None,
                 boundary_conditions="periodic", source_terms=None):
        from .semidiscretization import SemidiscretizationHyperbolicGPU
        from .solver import VolumeIntegralShockCapturingHG

        if not all(getattr(mesh, "periodicity", (True,))) or boundary_conditions not in ("periodic", None):
            raise NotImplementedError("partitioned runs support periodic TreeMeshes only")
        if source_terms is not None:
            raise NotImplementedError("partitioned runs support problems without source terms only")
        self.global_containers = mesh.build_containers(solver.basis.nodes)
        self.ranges = partition_ranges(self.global_containers.nelements, nranks)
        # shock capturing smooths the indicator with the ghosts' own values,
        # which need every node of a ghost
        mode = "elements" if isinstance(solver.volume_integral, VolumeIntegralShockCapturingHG) else "faces"
        self.part = build_local(self.global_containers, self.ranges, rank, mode=mode)
        self.semi = SemidiscretizationHyperbolicGPU(mesh, equations, initial_condition, solver,
                                                    precision=precision, device=device,
                                                    containers=self.part.containers)

    def local_state(self, u_global):
        """The local array (owned, then ghosts) gathered from a global state."""
        import torch

        ids = torch.as_tensor(np.concatenate([self.part.owned, self.part.ghosts]), device=u_global.device)
        return u_global.index_select(0, ids).contiguous()

    def stage(self, u_out, u_in, k, a, b, dt, t):
        from .semidiscretization import rk_stage

        rk_stage(u_out, u_in, k, a, b, dt, t, self.semi)

    def rk_steps(self, u_local, k_local, t, dt, nsteps, group=None):
        """nsteps CarpenterKennedy2N54 steps, one halo exchange before each
        stage; stage s runs at time t + c_s dt."""
        import torch

        from .time_integration import CK2N54_A, CK2N54_B, CK2N54_C

        other = torch.empty_like(u_local)
        cur, nxt = u_local, other
        for _ in range(nsteps):
            for a, b, c in zip(CK2N54_A, CK2N54_B, CK2N54_C):
                halo_exchange(cur.view(self.semi.u_shape()), self.part, group)
                self.stage(nxt, cur, k_local, a, b, dt, t + c * dt)
                cur, nxt = nxt, cur
            t += dt
        if cur is not u_local:
            u_local.copy_(cur)
        return u_local


def rk_steps_colocated(semis, u_locals, k_locals, t, dt, nsteps):
    """rk_steps of several PartitionedSemidiscretizationGPU ranks held in one
    process, in lockstep: before each stage every rank's ghost traces are
    refreshed by device copies (colocated_exchange), then every rank runs the
    stage."""
    import torch

    from .time_integration import CK2N54_A, CK2N54_B, CK2N54_C

    parts = [s_.part for s_ in semis]
    cur = list(u_locals)
    nxt = [torch.empty_like(u) for u in u_locals]
    for _ in range(nsteps):
        for a, b, c in zip(CK2N54_A, CK2N54_B, CK2N54_C):
            colocated_exchange([u.view(s_.semi.u_shape()) for u, s_ in zip(cur, semis)], parts)
            for i, s_ in enumerate(semis):
                s_.stage(nxt[i], cur[i], k_locals[i], a, b, dt, t + c * dt)
            cur, nxt = nxt, cur
        t += dt
    for u, c_ in zip(u_locals, cur):
        if c_ is not u:
            u.copy_(c_)
    return u_locals
