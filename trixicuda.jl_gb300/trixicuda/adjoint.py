"""Discrete adjoint of the GPU semidiscretization and of CarpenterKennedy2N54.

The reference has no differentiation capability.  Here the adjoint is exact
(up to round-off) for the discrete scheme: `rhs_vjp` applies J_rhs(u)^T with
hand-derived reverse-mode derivatives of the two-point fluxes, and
`AdjointSolve` reverses whole RK solves with binomial checkpointing
(Griewank-Walther "revolve" schedule) in libtrixi_b200.so.
`RKSolve` wraps it as a torch.autograd.Function -- the Python counterpart of a
ChainRulesCore `rrule` for the Julia side.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .semidiscretization import _call, _check_state, _stream_handle, _torch


def rhs_vjp(ubar, u, lam, semi, stream=None):
    """ubar = J_rhs(u)^T lam (all float64 CUDA tensors in the state layout)."""
    _check_state(semi, ubar, u, lam)
    _call(semi, semi._lib.trixi_rhs_vjp, C.c_void_p(ubar.data_ptr()), C.c_void_p(u.data_ptr()),
          C.c_void_p(lam.data_ptr()), stream=stream)


def objective_density_l2(u, rho_target, semi, grad=True, stream=None):
    """J = 1/2 int (rho - rho_target)^2 by LGL quadrature, and dJ/du."""
    torch = _torch()
    _check_state(semi, u)
    rt = rho_target.contiguous()
    if rt.numel() != semi.nelements * semi.nnodes ** semi.mesh.ndims or rt.dtype != torch.float64:
        raise ValueError("rho_target needs one float64 value per node")
    ubar = torch.empty_like(u) if grad else None
    J = C.c_double()
    _lib.check(semi._lib.trixi_objective_density_l2(
        semi._handle, C.c_void_p(u.data_ptr()), C.c_void_p(rt.data_ptr()), C.byref(J),
        C.c_void_p(ubar.data_ptr()) if grad else None, _stream_handle(stream)), semi._handle)
    return J.value, ubar


class AdjointSolve:
    """forward(u0) -> u(T) storing checkpoints; backward(dJ/du(T)) -> dJ/du0."""

    def __init__(self, semi, dt, nsteps, snapshots=15):
        self.semi, self.dt, self.nsteps, self.snapshots = semi, float(dt), int(nsteps), int(snapshots)
        self.forward_steps_recomputed = None

    def forward(self, u0, stream=None):
        torch = _torch()
        _check_state(self.semi, u0)
        uT = torch.empty_like(u0)
        _call(self.semi, self.semi._lib.trixi_adjoint_forward, C.c_void_p(u0.data_ptr()), self.dt, self.nsteps,
              self.snapshots, C.c_void_p(uT.data_ptr()), stream=stream)
        return uT

    def backward(self, uT_bar, stream=None):
        torch = _torch()
        _check_state(self.semi, uT_bar)
        u0_bar = torch.empty_like(uT_bar)
        n = C.c_int64()
        _call(self.semi, self.semi._lib.trixi_adjoint_backward, C.c_void_p(uT_bar.data_ptr()),
              C.c_void_p(u0_bar.data_ptr()), C.byref(n), stream=stream)
        self.forward_steps_recomputed = int(n.value)
        return u0_bar


def gradient_density_l2(semi, u0, rho_target, dt, nsteps, snapshots=15):
    """(J(u(T)), dJ/du0) for J = 1/2 int (rho(T) - rho_target)^2."""
    solve = AdjointSolve(semi, dt, nsteps, snapshots)
    uT = solve.forward(u0)
    J, uT_bar = objective_density_l2(uT, rho_target, semi)
    grad = solve.backward(uT_bar)
    return J, grad, solve.forward_steps_recomputed


def _make_autograd_function():
    torch = _torch()

    class RKSolve(torch.autograd.Function):
        """u(T) = RK solve of u0; backward = discrete adjoint (revolve checkpoints)."""

        @staticmethod
        def forward(ctx, u0, semi, dt, nsteps, snapshots=15):
            solve = AdjointSolve(semi, dt, nsteps, snapshots)
            ctx.solve = solve
            return solve.forward(u0.detach().contiguous())

        @staticmethod
        def backward(ctx, grad_out):
            return ctx.solve.backward(grad_out.contiguous()), None, None, None, None

    return RKSolve


def rk_solve_autograd(u0, semi, dt, nsteps, snapshots=15):
    return _make_autograd_function().apply(u0, semi, dt, nsteps, snapshots)
