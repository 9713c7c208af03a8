"""Independent TreeMesh connectivity for the oracle (test infrastructure).

TEST INFRASTRUCTURE ONLY.  The oracle builds the containers it computes on
itself, without the product package (trixicuda.mesh), so that a convention
error in the product's mesh code cannot hide inside both sides of a parity
test.  The construction is deliberately different from the product's tree
walk: every leaf is rasterised into a dense array over the finest level's
cells (`owner[i_1, .., i_d]` = leaf id), element order is a sort by the
Morton code of the leaf's lowest finest-level cell, and every face relation
is read off the raster one finest-level cell across the face.

Conventions restated from the reference's containers and kernels (and Trixi's
`TreeMesh` / `init_*`, which the reference calls, `src/solvers/cache.jl:60-88`):
* elements in depth-first order, children in Morton order with the x bit
  fastest (the order of Trixi's cell ids under uniform refinement);
* `interfaces.neighbor_ids[:, i] = (left, right)` along orientation i, one per
  +direction face between equal-size leaves, listed by element then direction
  (`src/solvers/containers_2d.jl:58`);
* L2 mortars listed by large element then direction (-x, +x, -y, ...):
  neighbor_ids = the small elements ordered by their position along the
  first, then the second tangential dimension, then the large element;
  large_side 1 when the large element is on the lower side
  (`src/solvers/dg_2d_kernel.jl:1371,1381`);
* boundaries: element faces on non-periodic domain faces, by direction
  (x_neg, x_pos, y_neg, ...) then element, neighbor_side 2 on a lower face;
* "box" refinement patches refine every leaf whose centre lies in the box,
  then coarse leaves are refined until face neighbours differ by at most one
  level (periodic wrap included).
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np


def _morton(coords, bits):
    """Morton code of integer cell coordinates (x bit fastest)."""
    d = len(coords)
    code = 0
    for b in range(bits):
        for k in range(d):
            code |= ((coords[k] >> b) & 1) << (b * d + k)
    return code


class OracleTreeMesh:
    """Leaves of a 2^d-tree over [coordinates_min, coordinates_max] (hypercube
    of side max(extent)), held as {(level, coords)}."""

    def __init__(self, coordinates_min, coordinates_max, initial_refinement_level, refinement_patches=(),
                 periodicity=True):
        self.cmin = np.atleast_1d(np.asarray(coordinates_min, dtype=np.float64))
        self.cmax = np.atleast_1d(np.asarray(coordinates_max, dtype=np.float64))
        self.d = d = self.cmin.size
        per = periodicity if isinstance(periodicity, (tuple, list)) else (periodicity,) * d
        self.periodic = tuple(bool(p) for p in per)
        self.L0 = float(np.max(self.cmax - self.cmin))
        self.lo = 0.5 * (self.cmin + self.cmax) - 0.5 * self.L0
        lvl = int(initial_refinement_level)
        n = 1 << lvl
        grid = np.stack(np.meshgrid(*([np.arange(n)] * d), indexing="ij"), axis=-1).reshape(-1, d)
        self.leaves = {(lvl, tuple(int(v) for v in c)) for c in grid}
        for patch in refinement_patches:
            if patch.get("type", "box") != "box":
                raise NotImplementedError("only box refinement patches")
            bmin = np.atleast_1d(np.asarray(patch["coordinates_min"], dtype=np.float64))
            bmax = np.atleast_1d(np.asarray(patch["coordinates_max"], dtype=np.float64))
            hit = [c for c in self.leaves if np.all(self.center(c) >= bmin) and np.all(self.center(c) <= bmax)]
            for c in hit:
                self._split(c)
            while self._balance_pass():
                pass
        self._rasterise()

    # -- geometry -------------------------------------------------------
    def length(self, cell):
        return self.L0 / (2 ** cell[0])

    def center(self, cell):
        return self.lo + (np.asarray(cell[1], dtype=np.float64) + 0.5) * self.length(cell)

    def _split(self, cell):
        lvl, c = cell
        self.leaves.remove(cell)
        for k in range(1 << self.d):
            self.leaves.add((lvl + 1, tuple(2 * c[j] + ((k >> j) & 1) for j in range(self.d))))

    # -- raster ---------------------------------------------------------
    def _raster(self):
        top = max(c[0] for c in self.leaves)
        n = 1 << top
        owner = np.full((n,) * self.d, -1, dtype=np.int64)
        level = np.zeros((n,) * self.d, dtype=np.int64)
        leaves = list(self.leaves)
        for i, (lvl, c) in enumerate(leaves):
            s = 1 << (top - lvl)
            sl = tuple(slice(ci * s, (ci + 1) * s) for ci in c)
            owner[sl] = i
            level[sl] = lvl
        assert np.all(owner >= 0), "leaves do not tile the domain"
        return top, owner, level, leaves

    def _across(self, top, cell, dim, side):
        """Finest-level cells across face (dim, side) of `cell`, as an index
        tuple of arrays, or None outside a non-periodic domain."""
        lvl, c = cell
        s = 1 << (top - lvl)
        n = 1 << top
        rng = [np.arange(ci * s, (ci + 1) * s) for ci in c]
        x = c[dim] * s + (s if side > 0 else -1)
        if not 0 <= x < n:
            if not self.periodic[dim]:
                return None
            x %= n
        rng[dim] = np.array([x])
        return np.ix_(*rng)

    def _balance_pass(self):
        top, owner, level, leaves = self._raster()
        split = set()
        for cell in leaves:
            for dim in range(self.d):
                for side in (-1, 1):
                    idx = self._across(top, cell, dim, side)
                    if idx is not None and int(level[idx].max()) > cell[0] + 1:
                        split.add(cell)
        for c in split:
            self._split(c)
        return bool(split)

    def _rasterise(self):
        top, owner, level, leaves = self._raster()
        for cell in leaves:
            for dim in range(self.d):
                for side in (-1, 1):
                    idx = self._across(top, cell, dim, side)
                    if idx is not None and abs(int(level[idx].max()) - cell[0]) > 1:
                        raise ValueError("mesh is not 2:1 balanced")
        keys = [_morton([ci << (top - lvl) for ci in c], top) for (lvl, c) in leaves]
        order = np.argsort(np.asarray(keys, dtype=np.int64), kind="stable")
        self.top = top
        self.elements = [leaves[i] for i in order]
        rank = np.empty(len(leaves), dtype=np.int64)
        rank[order] = np.arange(len(leaves))
        self.owner = rank[owner]  # raster of element ids (0-based, Morton order)

    # -- containers -----------------------------------------------------
    def containers(self, nodes):
        """init_elements / init_interfaces / init_mortars / init_boundaries
        restated on the raster, for LGL `nodes`."""
        d, top = self.d, self.top
        nodes = np.asarray(nodes, dtype=np.float64)
        N = nodes.size
        E = len(self.elements)
        inv_jac = np.empty(E)
        coords = np.empty((E,) + (N,) * d + (d,))
        for e, cell in enumerate(self.elements):
            h = self.length(cell)
            ctr = self.center(cell)
            inv_jac[e] = 2.0 / h
            for k in range(d):
                # memory order (E, N_z, .., N_x, d): the coordinate along k varies with index d-1-k
                shape = [1] * d
                shape[d - 1 - k] = N
                coords[e, ..., k] = np.broadcast_to((ctr[k] + 0.5 * h * nodes).reshape(shape), (N,) * d)
        if_nid, if_ori, mo_nid, mo_ls, mo_ori = [], [], [], [], []
        bnd = [[] for _ in range(2 * d)]
        for e, cell in enumerate(self.elements):
            lvl = cell[0]
            for dim in range(d):
                idx = self._across(top, cell, dim, +1)
                if idx is not None:
                    ids = np.unique(self.owner[idx])
                    if ids.size == 1 and self.elements[int(ids[0])][0] == lvl:
                        if_nid.append((e + 1, int(ids[0]) + 1))
                        if_ori.append(dim + 1)
            for direction in range(2 * d):
                dim, side = direction // 2, (1 if direction % 2 else -1)
                idx = self._across(top, cell, dim, side)
                if idx is None:
                    bnd[direction].append(e + 1)
                    continue
                block = self.owner[idx]
                if self.elements[int(block.flat[0])][0] != lvl + 1:
                    continue
                # small elements: quarter the face along the tangential dimensions
                tang = [t for t in range(d) if t != dim]
                half = (1 << (top - lvl)) // 2
                smalls = []
                for b2 in ((0, 1) if len(tang) > 1 else (0,)):
                    for b1 in ((0, 1) if tang else (0,)):
                        pos = [0] * d
                        if tang:
                            pos[tang[0]] = b1 * half
                        if len(tang) > 1:
                            pos[tang[1]] = b2 * half
                        smalls.append(int(block[tuple(pos)]) + 1)
                mo_nid.append(tuple(smalls) + (e + 1,))
                mo_ls.append(1 if side > 0 else 2)
                mo_ori.append(dim + 1)
        nc = 2 ** (d - 1)
        return SimpleNamespace(
            ndims=d, nnodes=N, nelements=E, inverse_jacobian=inv_jac, node_coordinates=coords,
            element_level=np.array([c[0] for c in self.elements], dtype=np.int64),
            interface_neighbor_ids=np.asarray(if_nid, dtype=np.int64).reshape(-1, 2),
            interface_orientations=np.asarray(if_ori, dtype=np.int64),
            mortar_neighbor_ids=np.asarray(mo_nid, dtype=np.int64).reshape(-1, nc + 1),
            mortar_large_sides=np.asarray(mo_ls, dtype=np.int64),
            mortar_orientations=np.asarray(mo_ori, dtype=np.int64),
            boundary_neighbor_ids=np.asarray([e for b in bnd for e in b], dtype=np.int64),
            boundary_neighbor_sides=np.asarray([2 if k % 2 == 0 else 1 for k in range(2 * d) for _ in bnd[k]],
                                               dtype=np.int64),
            boundary_orientations=np.asarray([k // 2 + 1 for k in range(2 * d) for _ in bnd[k]], dtype=np.int64),
            ninterfaces=len(if_ori), nmortars=len(mo_ori), nboundaries=sum(len(b) for b in bnd))
