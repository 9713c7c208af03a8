"""The benchmark workloads built from oracle code alone (test infrastructure).

TEST INFRASTRUCTURE ONLY.  bench.py's CPU leg (`cpu_baseline` and the
`--impl reference` arm) builds its problem here, so that it neither imports
the product package nor loads libtrixi_b200.so: the connectivity comes from
oracle/treemesh.py, the LGL basis from the oracle library, and the seeded
synthetic initial condition is restated below with the same definition and
random draws as the product's `initial_condition_fourier_euler` (a CPU test
checks that both give the same state).
"""
from __future__ import annotations

import numpy as np

from .oracle import EQ_EULER, FLUX_RANOCHA, VOL_FLUXDIFF, Oracle, basis
from .treemesh import OracleTreeMesh


def fourier_field(ndims, kmax, seed, xmin, xmax):
    """Seeded smooth periodic field on [xmin, xmax]^d: random normal
    coefficients on every integer wave vector 0 < |k| <= kmax (listed in
    lexicographic order of k + kmax), normalised by the sum of their
    magnitudes so that |field| <= 1."""
    rng = np.random.default_rng(seed)
    grid = np.indices((2 * kmax + 1,) * ndims).reshape(ndims, -1).T - kmax
    norm = np.sqrt(np.sum(grid * grid, axis=1))
    k = grid[(norm > 0) & (norm <= kmax)].astype(np.float64)
    a = rng.standard_normal(k.shape[0])
    b = rng.standard_normal(k.shape[0])
    s = np.sum(np.abs(a) + np.abs(b))
    a, b = a / s, b / s
    L = float(xmax) - float(xmin)

    def f(x):
        phase = 2 * np.pi * (k @ (x - float(xmin))) / L
        return a @ np.cos(phase) + b @ np.sin(phase)

    return f


def euler_fourier_state(coords, gamma=1.4, seed=20261203, kmax=8, xmin=-2.0, xmax=2.0, amplitude=0.1,
                        v0=(0.1, 0.2, 0.05), v_amp=0.02):
    """Conservative state [E, N.., nvars] of rho = 1 + amplitude F_0,
    v = v0 + v_amp F_{1..d}, p = 1 at the node coordinates [E, N.., d]."""
    d = coords.shape[-1]
    x = coords.reshape(-1, d).T
    rho = 1.0 + amplitude * fourier_field(d, kmax, seed, xmin, xmax)(x)
    v = np.stack([v0[i] + v_amp * fourier_field(d, kmax, seed + 1 + i, xmin, xmax)(x) for i in range(d)])
    u = np.empty((d + 2, rho.size))
    u[0] = rho
    u[1:1 + d] = rho * v
    u[-1] = 1.0 / (gamma - 1) + 0.5 * rho * np.sum(v * v, axis=0)
    return np.ascontiguousarray(u.T.reshape(coords.shape[:-1] + (d + 2,)))


def euler2d_fd_workload(level=7, polydeg=3, gamma=1.4, seed=20261203, kmax=8):
    """2D compressible Euler on [-2,2]^2 periodic at `level`, flux_ranocha
    volume and surface fluxes: (oracle, initial state, number of elements)."""
    mesh = OracleTreeMesh((-2.0, -2.0), (2.0, 2.0), level)
    cont = mesh.containers(basis(polydeg)["nodes"])
    orc = Oracle(cont, 2, polydeg, 4, EQ_EULER, gamma=gamma, volume_integral=VOL_FLUXDIFF,
                 volume_flux=FLUX_RANOCHA, surface_flux=FLUX_RANOCHA)
    u = euler_fourier_state(cont.node_coordinates, gamma, seed, kmax)
    return orc, u, cont.nelements
