"""Problem factories shared by the tests (mirroring the reference test files'
set-ups: test/tree_dgsem_{1,2,3}d/*.jl)."""
import numpy as np

import trixicuda as T

QUADRANT = {2: dict(type="box", coordinates_min=(0.0, 0.0), coordinates_max=(2.0, 2.0)),
            3: dict(type="box", coordinates_min=(0.0, 0.0, 0.0), coordinates_max=(2.0, 2.0, 2.0))}


def make(kind, ndims, level, polydeg=3, refined=False, precision="fp64", surface_flux=None, volume_flux=None,
         fv_flux=None, seed=1234, alpha_smooth=True):
    """kind: 'adv_weak', 'adv_fd', 'euler_fd', 'euler_weak', 'euler_sc'."""
    lo, hi = (-2.0, 2.0) if kind.startswith("euler") else (-1.0, 1.0)
    patches = []
    if refined:
        q = dict(QUADRANT[ndims])
        q["coordinates_min"] = tuple([lo * 0.0] * ndims)
        q["coordinates_max"] = tuple([hi] * ndims)
        patches = [q]
    mesh = T.TreeMesh((lo,) * ndims if ndims > 1 else lo, (hi,) * ndims if ndims > 1 else hi,
                      initial_refinement_level=level, refinement_patches=patches)
    if kind.startswith("adv"):
        a = (0.2, -0.7, 0.5)[:ndims] if ndims > 1 else (1.0,)
        cls = {1: T.LinearScalarAdvectionEquation1D, 2: T.LinearScalarAdvectionEquation2D,
               3: T.LinearScalarAdvectionEquation3D}[ndims]
        eq = cls(a)
        ic = T.initial_condition_convergence_test
        sf = surface_flux or T.flux_lax_friedrichs
        vi = T.VolumeIntegralWeakForm() if kind == "adv_weak" else T.VolumeIntegralFluxDifferencing(T.flux_central)
    else:
        cls = {1: T.CompressibleEulerEquations1D, 2: T.CompressibleEulerEquations2D,
               3: T.CompressibleEulerEquations3D}[ndims]
        eq = cls(1.4)
        if kind == "euler_sc":
            ic = T.initial_condition_weak_blast_wave
            ind = T.IndicatorHennemannGassner(eq, None, alpha_max=0.5, alpha_min=0.001, alpha_smooth=alpha_smooth)
            vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=volume_flux or T.flux_ranocha,
                                                  volume_flux_fv=fv_flux or T.flux_lax_friedrichs)
            sf = surface_flux or T.flux_lax_friedrichs
        else:
            ic = T.initial_condition_fourier_euler(eq, seed=seed, kmax=3, xmin=lo, xmax=hi)
            sf = surface_flux or T.flux_ranocha
            vi = (T.VolumeIntegralWeakForm() if kind == "euler_weak"
                  else T.VolumeIntegralFluxDifferencing(volume_flux or T.flux_ranocha))
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=sf, volume_integral=vi)
    return mesh, eq, ic, solver, precision


def semi_and_oracle(*args, **kw):
    from oracle.oracle import Oracle

    mesh, eq, ic, solver, precision = make(*args, **kw)
    semi = T.SemidiscretizationHyperbolicGPU(mesh, eq, ic, solver, precision=precision)
    return semi, Oracle.from_semi(semi)


def host_problem(*args, **kw):
    """Containers + oracle without touching the GPU."""
    from oracle.oracle import Oracle

    mesh, eq, ic, solver, precision = make(*args, **kw)
    cont = mesh.build_containers(solver.basis.nodes)

    class _S:
        pass

    s = _S()
    s.equations, s.solver, s.containers, s.mesh = eq, solver, cont, mesh
    s.initial_condition = ic
    orc = Oracle.from_semi(s)
    d = mesh.ndims
    x = cont.node_coordinates.reshape(-1, d).T
    u = ic(x, 0.0, eq).T.reshape((cont.nelements,) + (solver.polydeg + 1,) * d + (eq.nvariables,))
    return s, orc, np.ascontiguousarray(u)
