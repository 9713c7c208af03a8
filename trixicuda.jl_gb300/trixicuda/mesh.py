"""TreeMesh and its DG connectivity containers (host side).

Mirrors what the reference obtains from Trixi.jl's `TreeMesh` and
`init_elements` / `init_interfaces` / `init_mortars` before copying them to the
GPU (src/solvers/cache.jl:60-88, containers_{1,2,3}d.jl):

* a 2^d-tree over a hypercube; leaves are the DG elements, stored in
  depth-first order with children in Morton order (x bit fastest), which for
  uniform refinement is the order of Trixi's cell ids;
* `refinement_patches` of type "box" refine every leaf whose centre lies in
  the box (one extra level per patch); after each patch, coarser leaves are
  refined until every face neighbour differs by at most one level (2:1
  balance across faces, periodic wrap included), as Trixi's `refine!` keeps
  its trees;
* interfaces between equal-size neighbours: neighbor_ids[:, k] = (left,
  right) along orientation k (1-based), one interface per +direction face;
* L2 mortars where a leaf faces a refined neighbour: neighbor_ids = small
  elements (2D: lower, upper; 3D: lower_left, lower_right, upper_left,
  upper_right, with left/right along the first and lower/upper along the
  second tangential dimension) and then the large element; large_side 1
  means the large element is on the left (lower coordinate).

* boundaries (non-periodic dimensions): one entry per element face on the
  domain boundary, ordered by direction (x_neg, x_pos, y_neg, y_pos, z_neg,
  z_pos) and by element within a direction, with neighbor_sides 2 when the
  boundary is the element's lower face (the element lies on its right) and 1
  when it is the upper face -- the layout of Trixi's boundaries container.

Arrays are numpy arrays in C order whose memory layout equals the reference's
Julia column-major arrays: e.g. node_coordinates [ndims, N, N, E] is stored as
shape (E, N, N, ndims).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Containers:
    ndims: int
    nnodes: int
    nelements: int
    inverse_jacobian: np.ndarray            # (E,)
    node_coordinates: np.ndarray            # (E, N.., ndims)
    element_level: np.ndarray               # (E,)
    interface_neighbor_ids: np.ndarray      # (I, 2) int64, 1-based
    interface_orientations: np.ndarray      # (I,) int64, 1..ndims
    mortar_neighbor_ids: np.ndarray         # (M, 2^(d-1)+1) int64, 1-based
    mortar_large_sides: np.ndarray          # (M,)
    mortar_orientations: np.ndarray         # (M,)
    element_neighbors: dict = field(default_factory=dict)
    boundary_neighbor_ids: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))  # (B,) 1-based
    boundary_neighbor_sides: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))  # (B,) 1 or 2
    boundary_orientations: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))  # (B,) 1..ndims
    n_boundaries_per_direction: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int64))  # (2 ndims,)

    @property
    def nboundaries(self) -> int:
        return int(self.boundary_orientations.shape[0])

    @property
    def ninterfaces(self) -> int:
        return int(self.interface_orientations.shape[0])

    @property
    def nmortars(self) -> int:
        return int(self.mortar_orientations.shape[0])


class TreeMesh:
    """Hypercube 2^d-tree mesh (reference: Trixi.jl `TreeMesh`)."""

    def __init__(self, coordinates_min, coordinates_max, initial_refinement_level: int,
                 refinement_patches=(), n_cells_max: int | None = None, periodicity=True):
        cmin = np.atleast_1d(np.asarray(coordinates_min, dtype=np.float64))
        cmax = np.atleast_1d(np.asarray(coordinates_max, dtype=np.float64))
        if cmin.shape != cmax.shape:
            raise ValueError("coordinates_min/max dimension mismatch")
        self.ndims = int(cmin.shape[0])
        if self.ndims not in (1, 2, 3):
            raise ValueError("TreeMesh supports 1, 2, 3 dimensions")
        per = periodicity if isinstance(periodicity, (tuple, list)) else (periodicity,) * self.ndims
        if len(per) != self.ndims:
            raise ValueError("periodicity needs one flag per dimension")
        self.periodicity = tuple(bool(p) for p in per)
        self.length_level_0 = float(np.max(cmax - cmin))
        self.center_level_0 = 0.5 * (cmin + cmax)
        self.coordinates_min = cmin
        self.coordinates_max = cmax
        self.initial_refinement_level = int(initial_refinement_level)
        self.refinement_patches = [dict(p) for p in refinement_patches]
        # the tree: set of all cells and set of leaves, keyed (level, coords)
        root = (0, (0,) * self.ndims)
        self.cells = {root}
        self.leaves = {root}
        for _ in range(self.initial_refinement_level):
            for leaf in sorted(self.leaves):
                self._refine(leaf)
        for patch in refinement_patches:
            ptype = patch.get("type", "box")
            if ptype != "box":
                raise NotImplementedError(f"refinement patch type {ptype!r}")
            bmin = np.atleast_1d(np.asarray(patch["coordinates_min"], dtype=np.float64))
            bmax = np.atleast_1d(np.asarray(patch["coordinates_max"], dtype=np.float64))
            for leaf in sorted(self.leaves):
                c = self.cell_center(leaf)
                if np.all(c >= bmin) and np.all(c <= bmax):
                    self._refine(leaf)
            self._balance()
        if n_cells_max is not None and len(self.cells) > n_cells_max:
            raise ValueError(f"mesh needs {len(self.cells)} cells > n_cells_max={n_cells_max}")
        self._check_balance()
        self.elements = self._depth_first_leaves()
        self.element_index = {cell: i for i, cell in enumerate(self.elements)}

    # -- tree helpers ------------------------------------------------------
    def _children(self, cell):
        level, c = cell
        for bits in itertools.product((0, 1), repeat=self.ndims):
            bits = bits[::-1]  # x bit fastest (Morton order)
            yield (level + 1, tuple(2 * ci + b for ci, b in zip(c, bits)))

    def _refine(self, leaf):
        self.leaves.discard(leaf)
        for ch in self._children(leaf):
            self.cells.add(ch)
            self.leaves.add(ch)

    def _depth_first_leaves(self):
        out = []
        stack = [(0, (0,) * self.ndims)]
        while stack:
            cell = stack.pop()
            if cell in self.leaves:
                out.append(cell)
            else:
                stack.extend(reversed(list(self._children(cell))))
        return out

    def cell_length(self, cell) -> float:
        return self.length_level_0 / (2 ** cell[0])

    def cell_center(self, cell) -> np.ndarray:
        h = self.cell_length(cell)
        lo = self.center_level_0 - 0.5 * self.length_level_0
        return lo + (np.asarray(cell[1], dtype=np.float64) + 0.5) * h

    def _neighbor_cell(self, cell, dim, side):
        """The same-level cell across face (dim, side), or None beyond a
        non-periodic domain boundary."""
        level, c = cell
        n = 2 ** level
        cc = list(c)
        cc[dim] = cc[dim] + (1 if side > 0 else -1)
        if not 0 <= cc[dim] < n:
            if not self.periodicity[dim]:
                return None
            cc[dim] %= n
        return (level, tuple(cc))

    def _unbalanced(self, leaf):
        """True if a leaf face-neighbour of `leaf` is two or more levels finer."""
        for d in range(self.ndims):
            for side in (-1, 1):
                nb = self._neighbor_cell(leaf, d, side)
                if nb is not None and nb in self.cells and nb not in self.leaves:
                    for ch in self._face_children(nb, d, side):
                        if ch not in self.leaves:
                            return True
        return False

    def _balance(self):
        """Refine leaves until the mesh is 2:1 balanced across faces (the
        minimal such refinement; the result does not depend on the order)."""
        changed = True
        while changed:
            changed = False
            for leaf in sorted(self.leaves):
                if leaf in self.leaves and self._unbalanced(leaf):
                    self._refine(leaf)
                    changed = True

    def _check_balance(self):
        for leaf in self.leaves:
            for d in range(self.ndims):
                for side in (-1, 1):
                    nb = self._neighbor_cell(leaf, d, side)
                    if nb is not None and nb in self.cells and nb not in self.leaves:
                        for ch in self._face_children(nb, d, side):
                            if ch not in self.leaves:
                                raise ValueError("TreeMesh is not 2:1 balanced")

    def _face_children(self, nb, dim, side):
        """Children of refined cell nb adjacent to the face shared with a cell on
        the `-side` side, ordered (lower_left, lower_right, upper_left, upper_right)."""
        level, c = nb
        bit_d = 0 if side > 0 else 1
        tang = [d for d in range(self.ndims) if d != dim]
        out = []
        for b2 in ((0, 1) if len(tang) > 1 else (0,)):
            for b1 in ((0, 1) if len(tang) > 0 else (0,)):
                cc = [0] * self.ndims
                cc[dim] = 2 * c[dim] + bit_d
                if len(tang) > 0:
                    cc[tang[0]] = 2 * c[tang[0]] + b1
                if len(tang) > 1:
                    cc[tang[1]] = 2 * c[tang[1]] + b2
                out.append((level + 1, tuple(cc)))
        return out

    # -- public ------------------------------------------------------------
    @property
    def nelements(self) -> int:
        return len(self.elements)

    def ncells(self) -> int:
        return len(self.cells)

    def build_containers(self, nodes: np.ndarray) -> Containers:
        """init_elements / init_interfaces / init_mortars for LGL `nodes`."""
        d = self.ndims
        N = len(nodes)
        E = self.nelements
        inv_jac = np.empty(E)
        levels = np.empty(E, dtype=np.int64)
        coords = np.empty((E,) + (N,) * d + (d,))
        grids = np.meshgrid(*([nodes] * d), indexing="ij")  # grids[k][i0, i1, ...] = nodes[i_k]
        for e, cell in enumerate(self.elements):
            h = self.cell_length(cell)
            inv_jac[e] = 2.0 / h
            levels[e] = cell[0]
            ctr = self.cell_center(cell)
            for k in range(d):
                # memory order (E, N_z, N_y, N_x, ndims): transpose the ij grid
                coords[(e,) + (Ellipsis,) + (k,)] = (ctr[k] + 0.5 * h * grids[k]).transpose(tuple(range(d))[::-1])
        if_nid, if_ori = [], []
        mo_nid, mo_ls, mo_ori = [], [], []
        bnd = [[] for _ in range(2 * d)]  # per direction: element ids (1-based)
        for e, cell in enumerate(self.elements):
            for dim in range(d):
                nb = self._neighbor_cell(cell, dim, +1)
                if nb is not None and nb in self.leaves:
                    if_nid.append((e + 1, self.element_index[nb] + 1))
                    if_ori.append(dim + 1)
            for dir_ in range(2 * d):
                dim, side = dir_ // 2, (1 if dir_ % 2 else -1)
                nb = self._neighbor_cell(cell, dim, side)
                if nb is None:
                    bnd[dir_].append(e + 1)
                    continue
                if nb in self.cells and nb not in self.leaves:
                    smalls = [self.element_index[ch] + 1 for ch in self._face_children(nb, dim, side)]
                    mo_nid.append(tuple(smalls) + (e + 1,))
                    mo_ls.append(1 if side > 0 else 2)
                    mo_ori.append(dim + 1)
        nc = 2 ** (d - 1)
        b_nid = [e for dir_ in range(2 * d) for e in bnd[dir_]]
        b_side = [2 if dir_ % 2 == 0 else 1 for dir_ in range(2 * d) for _ in bnd[dir_]]
        b_ori = [dir_ // 2 + 1 for dir_ in range(2 * d) for _ in bnd[dir_]]
        return Containers(
            ndims=d, nnodes=N, nelements=E,
            inverse_jacobian=inv_jac,
            node_coordinates=coords,
            element_level=levels,
            interface_neighbor_ids=np.asarray(if_nid, dtype=np.int64).reshape(-1, 2),
            interface_orientations=np.asarray(if_ori, dtype=np.int64),
            mortar_neighbor_ids=np.asarray(mo_nid, dtype=np.int64).reshape(-1, nc + 1),
            mortar_large_sides=np.asarray(mo_ls, dtype=np.int64),
            mortar_orientations=np.asarray(mo_ori, dtype=np.int64),
            boundary_neighbor_ids=np.asarray(b_nid, dtype=np.int64),
            boundary_neighbor_sides=np.asarray(b_side, dtype=np.int64),
            boundary_orientations=np.asarray(b_ori, dtype=np.int64),
            n_boundaries_per_direction=np.asarray([len(b) for b in bnd], dtype=np.int64),
        )
