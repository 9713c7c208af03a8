"""Batched ensembles: hundreds of independent DGSEM problems advanced together
on one GPU (C ABI: trixi_batch_*).  The reference solves one problem at a
time; this is the batched mode of the GB300 library.

`BatchedSemidiscretizationGPU(problems)` takes a list of (mesh, equations,
initial_condition, solver) tuples, groups them by kernel kind inside the
library (one fused launch per group and RK stage, the whole step captured as
a CUDA graph), and exposes the batch state as one flat float64 CUDA tensor in
which instance i occupies a contiguous slice in its own reference layout.

`make_ensemble(...)` builds the seeded 512-instance mix of the batched
benchmark: 2D linear advection (levels 3-6), 2D compressible Euler with
flux_ranocha (levels 3-6) and 3D linear advection (levels 2-4), polydeg
uniform in 2..5, 25 % of the meshes with one quadrant/octant refined one
extra level (L2 mortars), smooth seeded Fourier initial conditions.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from . import equations as E
from .mesh import TreeMesh
from .semidiscretization import _check_state, _stream_handle, _torch, build_problem_desc
from .solver import DGSEMGPU, VolumeIntegralFluxDifferencing, VolumeIntegralWeakForm


def _batch_check(status, batch=None):
    if status != _lib.TRIXI_OK:
        buf = C.create_string_buffer(1024)
        _lib.load().trixi_batch_last_error(batch, buf, len(buf))
        raise _lib.TrixiError(status, buf.value.decode(errors="replace"))


@dataclass
class Problem:
    mesh: TreeMesh
    equations: object
    initial_condition: object
    solver: DGSEMGPU
    label: str = ""


class BatchedSemidiscretizationGPU:
    def __init__(self, problems, precision: str = "fp64", device=None):
        torch = _torch()
        self.problems = list(problems)
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self._keep = []
        self.containers = []
        cache = {}
        descs = []
        for pb in self.problems:
            key = (id(pb.mesh), pb.solver.polydeg)
            if key not in cache:
                cache[key] = pb.mesh.build_containers(pb.solver.basis.nodes)
            cont = cache[key]
            d, keep, _ = build_problem_desc(cont, pb.equations, pb.solver, precision)
            self._keep.append((d, keep))
            self.containers.append(cont)
            descs.append(d)
        arr = (C.POINTER(_lib.ProblemDesc) * len(descs))(*[C.pointer(d) for d in descs])
        lib = _lib.load()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _batch_check(lib.trixi_batch_create(arr, len(descs), C.byref(h)))
        self._h = h
        self._lib = lib
        n = len(descs)
        off = (C.c_int64 * n)()
        nv = (C.c_int64 * n)()
        tot = C.c_int64()
        ng = C.c_int64()
        _batch_check(lib.trixi_batch_layout(h, off, nv, C.byref(tot), C.byref(ng)), h)
        self.value_offsets = np.array(off[:], dtype=np.int64)
        self.nvalues = np.array(nv[:], dtype=np.int64)
        self.total_values = int(tot.value)
        self.ngroups = int(ng.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.trixi_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def __len__(self):
        return len(self.problems)

    def shape(self, i):
        pb = self.problems[i]
        return (self.containers[i].nelements,) + (pb.solver.polydeg + 1,) * pb.mesh.ndims + (pb.equations.nvariables,)

    def view(self, u, i):
        """Instance i of the flat batch state, shaped (nelements, N, .., nvars)."""
        o, n = int(self.value_offsets[i]), int(self.nvalues[i])
        return u[o:o + n].view(self.shape(i))

    def ndofs(self) -> int:
        return int(sum(c.nelements * (pb.solver.polydeg + 1) ** pb.mesh.ndims
                       for c, pb in zip(self.containers, self.problems)))

    def compute_coefficients(self):
        """The batch state with every instance's initial condition (evaluated
        on the GPU with torch for the Fourier fields, on the host otherwise)."""
        torch = _torch()
        u = torch.empty(self.total_values, dtype=torch.float64, device=self.device)
        for i, pb in enumerate(self.problems):
            x = torch.from_numpy(self.containers[i].node_coordinates.reshape(-1, pb.mesh.ndims).T.copy()).to(self.device)
            vals = pb.initial_condition(x, 0.0, pb.equations)
            if not isinstance(vals, torch.Tensor):
                vals = torch.from_numpy(np.asarray(vals)).to(self.device)
            self.view(u, i).copy_(vals.T.reshape(self.shape(i)))
        return u

    def rhs(self, du, u, stream=None):
        torch = _torch()
        for t in (du, u):
            if t.dtype != torch.float64 or not t.is_cuda or t.numel() != self.total_values:
                raise ValueError("batch state must be a float64 CUDA tensor of total_values")
        _batch_check(self._lib.trixi_batch_rhs(self._h, C.c_void_p(du.data_ptr()), C.c_void_p(u.data_ptr()),
                                               _stream_handle(stream)), self._h)

    def rk_steps(self, u, k, dt, nsteps, use_graph=True, stream=None):
        dt = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, dtype=np.float64), (len(self),)))
        _batch_check(self._lib.trixi_batch_rk_steps(self._h, C.c_void_p(u.data_ptr()), C.c_void_p(k.data_ptr()),
                                                    dt.ctypes.data_as(C.POINTER(C.c_double)), int(nsteps),
                                                    int(bool(use_graph)), _stream_handle(stream)), self._h)

    def tuning(self):
        """(chosen branch count, {candidate branch count: ms per step}) of the
        step-graph tuner; (0, {}) before the first graph build."""
        br = C.c_int()
        cand = (C.c_int * 16)()
        ms = (C.c_double * 16)()
        cnt = C.c_int64()
        _batch_check(self._lib.trixi_batch_tuning(self._h, C.byref(br), cand, ms, 16, C.byref(cnt)), self._h)
        n = min(int(cnt.value), 16)
        return int(br.value), {int(cand[i]): float(ms[i]) for i in range(n)}

    def group_of(self, i):
        """Group index of instance i: kinds are numbered in order of first
        appearance, as the library numbers them."""
        if not hasattr(self, "_group_index"):
            order, idx = {}, []
            for pb in self.problems:
                vi = pb.solver.volume_integral
                key = (pb.mesh.ndims, pb.solver.polydeg, type(pb.equations).__name__, type(vi).__name__,
                       repr(getattr(vi, "volume_flux", None)), repr(pb.solver.surface_flux))
                idx.append(order.setdefault(key, len(order)))
            self._group_index = idx
        return self._group_index[i]

    def group_tiles(self):
        """Per group: ((elements per group, warps per group, groups per block),
        the tile tuner's {(wpg, gpb): ms}) after the first graph build."""
        from .semidiscretization import _read_tile

        out = []
        for g in range(self.ngroups):
            h = C.c_void_p()
            _batch_check(self._lib.trixi_batch_handle(self._h, g, C.byref(h)), self._h)
            out.append(_read_tile(self._lib, h))
        return out

    def stable_dt(self, u, cfl=0.5):
        """Per-instance CFL time step cfl * 2 / (N * max J^{-1} sum_d lambda_d)."""
        torch = _torch()
        dts = np.empty(len(self))
        for i, pb in enumerate(self.problems):
            ui = self.view(u, i).reshape(-1, pb.equations.nvariables)
            d = pb.mesh.ndims
            if pb.equations.nvariables == 1:
                lam = float(np.sum(np.abs(pb.equations.advection_velocity)))
            else:
                rho = ui[:, 0]
                v = ui[:, 1:1 + d] / rho[:, None]
                p = (pb.equations.gamma - 1) * (ui[:, -1] - 0.5 * rho * torch.sum(v * v, dim=1))
                c = torch.sqrt(pb.equations.gamma * p / rho)
                lam = float(torch.max(torch.sum(torch.abs(v), dim=1) + d * c))
            ij = float(np.max(self.containers[i].inverse_jacobian))
            dts[i] = cfl * 2.0 / ((pb.solver.polydeg + 1) * ij * lam)
        return dts


class TorchFourierField:
    """E.FourierField evaluated on the GPU in chunks (same seeded modes)."""

    def __init__(self, ff: E.FourierField, device):
        torch = _torch()
        self.k = torch.from_numpy(ff.k).to(device)
        self.a = torch.from_numpy(ff.a).to(device)
        self.b = torch.from_numpy(ff.b).to(device)
        self.xmin, self.L = ff.xmin, ff.L

    def __call__(self, x):
        torch = _torch()
        out = torch.empty(x.shape[1], dtype=torch.float64, device=x.device)
        chunk = max(1, (1 << 26) // max(1, self.k.shape[0]))
        for s in range(0, x.shape[1], chunk):
            ph = (2 * np.pi / self.L) * (self.k @ (x[:, s:s + chunk] - self.xmin))
            out[s:s + chunk] = self.a @ torch.cos(ph) + self.b @ torch.sin(ph)
        return out


def _fourier_ic(eq, seed, kmax, xmin, xmax, device, amplitude=0.1, v0=(0.1, 0.2, 0.05), v_amp=0.02):
    torch = _torch()
    d = eq.ndims
    f0 = TorchFourierField(E.FourierField(d, kmax, seed, xmin, xmax), device)
    if eq.nvariables == 1:
        return lambda x, t, e: (1.0 + amplitude * f0(x))[None, :]
    fv = [TorchFourierField(E.FourierField(d, kmax, seed + 1 + i, xmin, xmax), device) for i in range(d)]

    def ic(x, t, e):
        rho = 1.0 + amplitude * f0(x)
        v = torch.stack([v0[i] + v_amp * fv[i](x) for i in range(d)])
        p = torch.ones_like(rho)
        u = torch.empty((e.nvariables,) + rho.shape, dtype=torch.float64, device=x.device)
        u[0] = rho
        u[1:1 + d] = rho * v
        u[-1] = p / (e.gamma - 1) + 0.5 * rho * torch.sum(v * v, dim=0)
        return u

    return ic


def make_ensemble(n=512, seed=20261203, kmax=8, device=None, refined_fraction=0.25):
    """The seeded batched-benchmark mix (see the module docstring)."""
    torch = _torch()
    device = device or torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(seed)
    meshes = {}
    problems = []
    for i in range(n):
        family = int(rng.integers(3))
        polydeg = int(rng.integers(2, 6))
        refined = bool(rng.random() < refined_fraction)
        if family == 2:
            d, level = 3, int(rng.integers(2, 5))
        else:
            d, level = 2, int(rng.integers(3, 7))
        lo, hi = (-2.0, 2.0) if family == 1 else (-1.0, 1.0)
        key = (d, level, refined, lo)
        if key not in meshes:
            patches = [dict(type="box", coordinates_min=(0.0,) * d, coordinates_max=(hi,) * d)] if refined else []
            meshes[key] = TreeMesh((lo,) * d, (hi,) * d, initial_refinement_level=level, refinement_patches=patches)
        mesh = meshes[key]
        if family == 1:
            eq = E.CompressibleEulerEquations2D(1.4)
            solver = DGSEMGPU(polydeg=polydeg, surface_flux=E.flux_ranocha,
                              volume_integral=VolumeIntegralFluxDifferencing(E.flux_ranocha))
        else:
            eq = (E.LinearScalarAdvectionEquation2D((0.2, -0.7)) if d == 2
                  else E.LinearScalarAdvectionEquation3D((0.2, -0.7, 0.5)))
            solver = DGSEMGPU(polydeg=polydeg, surface_flux=E.flux_lax_friedrichs,
                              volume_integral=VolumeIntegralWeakForm())
        ic = _fourier_ic(eq, seed + 7919 * i, kmax if d == 2 else min(kmax, 4), lo, hi, device)
        label = f"{['adv2d', 'euler2d', 'adv3d'][family]}-L{level}-p{polydeg}{'-ref' if refined else ''}"
        problems.append(Problem(mesh, eq, ic, solver, label))
    return problems
