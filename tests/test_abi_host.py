"""C ABI: the library loads, exports every entry point declared in
include/trixi_b200.h, and its host-side validation rejects bad input with
the documented status codes -- all without touching a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from trixicuda import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "trixi_b200.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(trixi_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load(build_if_missing=True)
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"


def test_version():
    lib = _lib.load()
    assert lib.trixi_version().decode().startswith("trixi_b200")
    assert lib.trixi_abi_version() == 1


def test_struct_size_matches_c():
    # the C struct size is checked by trixi_create; a mismatch is INVALID_ARGUMENT
    lib = _lib.load()
    d = _lib.ProblemDesc()
    d.struct_size = 12
    h = C.c_void_p()
    st = lib.trixi_create(C.byref(d), C.byref(h))
    assert st == 1 and "struct_size" in _lib.last_error()


def _desc_from_mesh(level=2, polydeg=3):
    import trixicuda as T
    from trixicuda.semidiscretization import build_problem_desc

    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEMGPU(polydeg=polydeg, surface_flux=T.flux_ranocha,
                        volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_ranocha))
    mesh = T.TreeMesh((-2, -2), (2, 2), initial_refinement_level=level)
    return build_problem_desc(mesh, eq, solver)


def _create(d):
    h = C.c_void_p()
    st = _lib.load().trixi_create(C.byref(d), C.byref(h))
    return st, _lib.last_error()


@pytest.mark.parametrize("field,value,status", [
    ("ndims", 4, 1), ("polydeg", 9, 2), ("nvars", 3, 1), ("equation", 7, 1),
    ("volume_integral", 5, 1), ("surface_flux", 9, 1), ("precision", 3, 1), ("nboundaries", 4, 1),
    ("source_terms", 3, 1), ("nboundary_params", 9, 1),
    ("gamma", 1.0, 1), ("nelements", 0, 1),
])
def test_create_rejects_bad_fields(field, value, status):
    d, keep, _ = _desc_from_mesh()
    setattr(d, field, value)
    st, msg = _create(d)
    assert st == status, msg
    assert msg


def test_create_rejects_bad_boundaries():
    import trixicuda as T
    from trixicuda.semidiscretization import build_problem_desc

    # a boundary declared on a face that a (periodic) interface already connects
    d, keep, _ = _desc_from_mesh()
    keep["fake_b"] = np.array([1], dtype=np.int64)
    ptr = keep["fake_b"].ctypes.data_as(C.POINTER(C.c_int64))
    d.nboundaries, d.boundary_function = 1, 1
    d.boundary_neighbor_ids = d.boundary_neighbor_sides = d.boundary_orientations = ptr
    st, msg = _create(d)
    assert st == 7 and "already connected" in msg
    # a non-periodic mesh needs a boundary function, and each boundary face a declaration
    eq = T.CompressibleEulerEquations2D(1.4)
    solver = T.DGSEMGPU(polydeg=2)
    mesh = T.TreeMesh((0, 0), (2, 2), initial_refinement_level=2, periodicity=False)
    bc = T.BoundaryConditionDirichlet(T.initial_condition_convergence_test)
    d, keep, _ = build_problem_desc(mesh, eq, solver, boundary_conditions=bc)
    d.boundary_function = 7
    st, msg = _create(d)
    assert st == 1 and "boundary_function" in msg
    d, keep, _ = build_problem_desc(mesh, eq, solver, boundary_conditions=bc)
    d.nboundaries = d.nboundaries - 1
    st, msg = _create(d)
    assert st == 7 and "no interface, mortar or boundary" in msg
    # the convergence-test source is defined for the Euler equations only
    adv = T.LinearScalarAdvectionEquation2D((1.0, 1.0))
    d, keep, _ = build_problem_desc(mesh, adv, solver, boundary_conditions=bc)
    d.source_terms = 1
    st, msg = _create(d)
    assert st == 2 and "Euler" in msg


def test_create_rejects_corrupted_connectivity():
    d, keep, _ = _desc_from_mesh()
    keep["if_nid"][3, 1] = 10_000          # neighbour id out of range
    st, msg = _create(d)
    assert st == 7 and "out of range" in msg
    d, keep, _ = _desc_from_mesh()
    keep["if_nid"][5] = keep["if_nid"][4]  # duplicated interface -> face connected twice
    st, msg = _create(d)
    assert st == 7 and "already connected" in msg
    d, keep, _ = _desc_from_mesh()
    d.ninterfaces = d.ninterfaces - 1      # a face left open (non-periodic)
    st, msg = _create(d)
    assert st == 7 and "has no interface" in msg
    d, keep, _ = _desc_from_mesh()
    keep["if_ori"][0] = 3                  # orientation out of range in 2D
    st, msg = _create(d)
    assert st == 7


def test_null_arguments():
    lib = _lib.load()
    assert lib.trixi_create(None, None) == 1
    assert lib.trixi_rhs(None, None, None, 0.0, None) == 1
    assert lib.trixi_rk_steps_host(None, None, None, 0.0, 1e-3, 1, None, None, None) == 1
    assert lib.trixi_destroy(None) == 0
    buf = C.create_string_buffer(4)
    lib.trixi_last_error(None, buf, 4)
    assert len(buf.value) <= 3  # truncated and NUL-terminated


def test_lgl_basis_entry_point_rejects_bad_input():
    lib = _lib.load()
    out = np.zeros(4)
    assert lib.trixi_lgl_basis(0, 0, out.ctypes.data_as(C.POINTER(C.c_double)), 4) == 1
    assert lib.trixi_lgl_basis(3, 2, out.ctypes.data_as(C.POINTER(C.c_double)), 4) == 1  # 16 needed
    assert lib.trixi_lgl_basis(3, 0, out.ctypes.data_as(C.POINTER(C.c_double)), 4) == 0


def _mhd_desc(d=2):
    import trixicuda as T
    from trixicuda.semidiscretization import build_problem_desc

    eq = {1: T.IdealGlmMhdEquations1D, 2: T.IdealGlmMhdEquations2D, 3: T.IdealGlmMhdEquations3D}[d](1.4, 1.0)
    pair = (lambda f: (f, T.flux_nonconservative_powell)) if d > 1 else (lambda f: f)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=pair(T.flux_lax_friedrichs),
                        volume_integral=T.VolumeIntegralFluxDifferencing(pair(T.flux_hindenlang_gassner)))
    mesh = T.TreeMesh((-2.0,) * d, (2.0,) * d, initial_refinement_level=1)
    return build_problem_desc(mesh, eq, solver)


@pytest.mark.parametrize("field,value,status", [
    ("nvars", 8, 1),                    # 2D ideal GLM-MHD has 9 variables
    ("nonconservative_flux", 0, 1),     # and needs flux_nonconservative_powell
    ("volume_flux", 1, 1),              # flux_ranocha is the Euler flux
    ("surface_flux", 5, 2),             # flux_shima_etal is a volume flux
    ("volume_integral", 0, 2),          # weak form with nonconservative terms
    ("polydeg", 5, 2),                  # the MHD kernels stop at polydeg 4
    ("source_terms", 1, 2),             # no source terms for MHD
])
def test_create_rejects_bad_mhd_fields(field, value, status):
    d, keep, _ = _mhd_desc()
    setattr(d, field, value)
    st, msg = _create(d)
    assert st == status, (field, st, msg)
    assert msg


@pytest.mark.parametrize("field,value,status", [
    ("nonconservative_flux", 1, 1),     # Euler has no nonconservative terms
    ("volume_flux", 4, 1),              # flux_hindenlang_gassner is the MHD flux
    ("surface_flux", 5, 2),             # flux_shima_etal as a surface flux
    ("volume_flux_fv", 5, 2),           # ... or as the FV flux
    ("surface_flux", 8, 1),             # no such flux
    ("volume_flux", 7, 2),              # flux_hlle as a volume flux
])
def test_create_rejects_bad_flux_pairs(field, value, status):
    d, keep, _ = _desc_from_mesh()
    setattr(d, field, value)
    st, msg = _create(d)
    assert st == status, (field, st, msg)


def test_mhd_boundary_rules():
    """Ideal GLM-MHD takes Dirichlet boundaries; a constant state of 9
    variables does not fit the descriptor's 8 boundary parameters and is
    refused, in Python before the call and by the library."""
    import trixicuda as T
    from trixicuda.semidiscretization import build_problem_desc

    eq = T.IdealGlmMhdEquations2D(1.4, 1.0)
    pair = lambda f: (f, T.flux_nonconservative_powell)  # noqa: E731
    solver = T.DGSEMGPU(polydeg=3, surface_flux=pair(T.flux_lax_friedrichs),
                        volume_integral=T.VolumeIntegralFluxDifferencing(pair(T.flux_hindenlang_gassner)))
    mesh = T.TreeMesh((0.0, 0.0), (2.0, 2.0), initial_refinement_level=1, periodicity=False)
    with pytest.raises(NotImplementedError):
        build_problem_desc(mesh, eq, solver,
                           boundary_conditions=T.BoundaryConditionDirichlet(T.initial_condition_constant))
    d, keep, _ = build_problem_desc(mesh, eq, solver,
                                    boundary_conditions=T.BoundaryConditionDirichlet(T.initial_condition_weak_blast_wave))
    assert d.nboundaries > 0 and d.boundary_function == 2
    d.boundary_function = 0
    st, msg = _create(d)
    assert st == 2 and "8 parameters" in msg
    d.boundary_function, d.source_terms = 2, 1
    st, msg = _create(d)
    assert st == 2 and "source" in msg


def test_create_rejects_bad_indicator_variable():
    import trixicuda as T
    from trixicuda.semidiscretization import build_problem_desc

    eq = T.CompressibleEulerEquations2D(1.4)
    ind = T.IndicatorHennemannGassner(eq, None)
    vi = T.VolumeIntegralShockCapturingHG(ind, volume_flux_dg=T.flux_ranocha, volume_flux_fv=T.flux_lax_friedrichs)
    solver = T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs, volume_integral=vi)
    d, keep, _ = build_problem_desc(T.TreeMesh((-1.0, -1.0), (1.0, 1.0), initial_refinement_level=1), eq, solver)
    d.indicator_variable = 2
    st, msg = _create(d)
    assert st == 1 and "indicator_variable" in msg


def test_flux_pairs_checked_on_the_host():
    """Plain fluxes for MHD in 2D, or pairs for Euler, are refused before the
    library is called."""
    import trixicuda as T
    from trixicuda.semidiscretization import flux_codes

    eq = T.IdealGlmMhdEquations2D(1.4)
    with pytest.raises(ValueError):
        flux_codes(T.DGSEMGPU(polydeg=3, surface_flux=T.flux_lax_friedrichs,
                              volume_integral=T.VolumeIntegralFluxDifferencing(T.flux_hindenlang_gassner)), eq)
    with pytest.raises(ValueError):
        flux_codes(T.DGSEMGPU(polydeg=3, surface_flux=(T.flux_ranocha, T.flux_nonconservative_powell)),
                   T.CompressibleEulerEquations2D(1.4))
