"""ctypes binding of libtrixi_b200.so (the C ABI declared in include/trixi_b200.h).

This is the Python counterpart of the `ccall` glue a Julia maintainer adds to
TrixiCUDA.jl (julia/TrixiGB300.jl).  The library is loaded from the in-tree
build folder; if it is missing the import fails loudly -- there is no CPU or
PyTorch fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build

TRIXI_OK = 0
STATUS_NAMES = {
    0: "TRIXI_OK",
    1: "TRIXI_ERR_INVALID_ARGUMENT",
    2: "TRIXI_ERR_UNSUPPORTED",
    3: "TRIXI_ERR_CUDA",
    4: "TRIXI_ERR_DEVICE_FLAG",
    5: "TRIXI_ERR_TIMEOUT",
    6: "TRIXI_ERR_OUT_OF_MEMORY",
    7: "TRIXI_ERR_BAD_CONNECTIVITY",
}

EQ_LINEAR_ADVECTION, EQ_COMPRESSIBLE_EULER, EQ_IDEAL_GLM_MHD = 0, 1, 2
VOLUME_WEAK_FORM, VOLUME_FLUX_DIFFERENCING, VOLUME_SHOCK_CAPTURING_HG = 0, 1, 2
FLUX_LAX_FRIEDRICHS, FLUX_RANOCHA, FLUX_CENTRAL, FLUX_LAX_FRIEDRICHS_NAIVE = 0, 1, 2, 3
FLUX_HINDENLANG_GASSNER = 4
FLUX_SHIMA_ETAL, FLUX_HLL, FLUX_HLLE = 5, 6, 7
NONCONSERVATIVE_NONE, NONCONSERVATIVE_POWELL = 0, 1
PRECISION_FP64, PRECISION_MIXED = 0, 1

IC_CONSTANT, IC_CONVERGENCE_TEST, IC_WEAK_BLAST_WAVE, IC_EOC_TEST_COUPLED_EULER_GRAVITY = 0, 1, 2, 3
SOURCE_NONE, SOURCE_CONVERGENCE_TEST, SOURCE_EOC_TEST_EULER = 0, 1, 2
INTEGRAL_STATE, INTEGRAL_ENTROPY, INTEGRAL_ENTROPY_PRODUCTION, INTEGRAL_DU = 0, 1, 2, 3

CONTAINER_INTERFACES_U = 0
CONTAINER_SURFACE_FLUX_VALUES = 1
CONTAINER_MORTARS_U = 2
CONTAINER_ALPHA = 8
CONTAINER_INVERSE_JACOBIAN = 9
CONTAINER_BOUNDARIES_U = 10

BASIS_ITEMS = {
    "nodes": 0, "weights": 1, "derivative_split": 2, "derivative_dhat": 3,
    "inverse_vandermonde_legendre": 4, "forward_upper": 5, "forward_lower": 6,
    "reverse_upper": 7, "reverse_lower": 8, "derivative_matrix": 9,
}


class TrixiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class ProblemDesc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_int32),
        ("ndims", C.c_int32),
        ("polydeg", C.c_int32),
        ("nvars", C.c_int32),
        ("equation", C.c_int32),
        ("volume_integral", C.c_int32),
        ("volume_flux", C.c_int32),
        ("surface_flux", C.c_int32),
        ("volume_flux_fv", C.c_int32),
        ("precision", C.c_int32),
        ("gamma", C.c_double),
        ("advection_velocity", C.c_double * 3),
        ("alpha_max", C.c_double),
        ("alpha_min", C.c_double),
        ("alpha_smooth", C.c_int32),
        ("indicator_variable", C.c_int32),
        ("nelements", C.c_int64),
        ("inverse_jacobian", C.POINTER(C.c_double)),
        ("ninterfaces", C.c_int64),
        ("interface_neighbor_ids", C.POINTER(C.c_int64)),
        ("interface_orientations", C.POINTER(C.c_int64)),
        ("nboundaries", C.c_int64),
        ("nmortars", C.c_int64),
        ("mortar_neighbor_ids", C.POINTER(C.c_int64)),
        ("mortar_large_sides", C.POINTER(C.c_int64)),
        ("mortar_orientations", C.POINTER(C.c_int64)),
        ("weights", C.POINTER(C.c_double)),
        ("derivative_split", C.POINTER(C.c_double)),
        ("derivative_dhat", C.POINTER(C.c_double)),
        ("inverse_vandermonde_legendre", C.POINTER(C.c_double)),
        ("forward_upper", C.POINTER(C.c_double)),
        ("forward_lower", C.POINTER(C.c_double)),
        ("reverse_upper", C.POINTER(C.c_double)),
        ("reverse_lower", C.POINTER(C.c_double)),
        ("node_coordinates", C.POINTER(C.c_double)),
        ("nghost_elements", C.c_int64),
        ("boundary_neighbor_ids", C.POINTER(C.c_int64)),
        ("boundary_neighbor_sides", C.POINTER(C.c_int64)),
        ("boundary_orientations", C.POINTER(C.c_int64)),
        ("boundary_function", C.c_int32),
        ("source_terms", C.c_int32),
        ("nboundary_params", C.c_int32),
        ("nsource_params", C.c_int32),
        ("boundary_params", C.c_double * 8),
        ("source_params", C.c_double * 3),
        ("nonconservative_flux", C.c_int32),
        ("reserved0", C.c_int32),
        ("glm_speed", C.c_double),
    ]


# (name, restype, argtypes) of every exported entry point
_VP, _DP, _I64, _D, _I = C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_int
SIGNATURES = {
    "trixi_version": (C.c_char_p, []),
    "trixi_abi_version": (C.c_int, []),
    "trixi_create": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)]),
    "trixi_destroy": (C.c_int, [_VP]),
    "trixi_last_error": (C.c_int, [_VP, C.c_char_p, C.c_size_t]),
    "trixi_rhs": (C.c_int, [_VP, _DP, _DP, _D, _VP]),
    "trixi_rk_stage": (C.c_int, [_VP, _DP, _DP, _DP, _D, _D, _D, _D, _VP]),
    "trixi_rk_steps": (C.c_int, [_VP, _DP, _DP, _D, _D, _I64, _VP]),
    "trixi_rk_steps_host": (C.c_int, [_VP, _DP, _DP, _D, _D, _I64, _VP, _VP, _VP]),
    "trixi_volume_integral": (C.c_int, [_VP, _DP, _DP, _VP]),
    "trixi_prolong2interfaces": (C.c_int, [_VP, _DP, _VP]),
    "trixi_interface_flux": (C.c_int, [_VP, _VP]),
    "trixi_prolong2boundaries": (C.c_int, [_VP, _DP, _VP]),
    "trixi_boundary_flux": (C.c_int, [_VP, _D, _VP]),
    "trixi_prolong2mortars": (C.c_int, [_VP, _DP, _VP]),
    "trixi_mortar_flux": (C.c_int, [_VP, _VP]),
    "trixi_surface_integral": (C.c_int, [_VP, _DP, _VP]),
    "trixi_jacobian": (C.c_int, [_VP, _DP, _VP]),
    "trixi_sources": (C.c_int, [_VP, _DP, _DP, _D, _VP]),
    "trixi_container": (C.c_int, [_VP, _I, C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
    "trixi_indicator": (C.c_int, [_VP, _DP, _DP, _VP]),
    "trixi_basis": (C.c_int, [_VP, _I, C.POINTER(C.c_double), _I64]),
    "trixi_lgl_basis": (C.c_int, [_I, _I, C.POINTER(C.c_double), _I64]),
    "trixi_synchronize": (C.c_int, [_VP, _VP]),
    "trixi_compute_coefficients": (C.c_int, [_VP, _I, C.POINTER(C.c_double), _I64, _D, _DP, _VP]),
    "trixi_max_dt": (C.c_int, [_VP, _DP, _DP, _VP]),
    "trixi_rhs_vjp": (C.c_int, [_VP, _DP, _DP, _DP, _VP]),
    "trixi_objective_density_l2": (C.c_int, [_VP, _DP, _DP, C.POINTER(C.c_double), _DP, _VP]),
    "trixi_adjoint_forward": (C.c_int, [_VP, _DP, _D, _I64, _I64, _DP, _VP]),
    "trixi_adjoint_backward": (C.c_int, [_VP, _DP, _DP, C.POINTER(C.c_int64), _VP]),
    "trixi_batch_create": (C.c_int, [C.POINTER(C.POINTER(ProblemDesc)), _I64, C.POINTER(C.c_void_p)]),
    "trixi_batch_destroy": (C.c_int, [_VP]),
    "trixi_batch_layout": (C.c_int, [_VP, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                     C.POINTER(C.c_int64)]),
    "trixi_batch_rhs": (C.c_int, [_VP, _DP, _DP, _VP]),
    "trixi_batch_rk_steps": (C.c_int, [_VP, _DP, _DP, C.POINTER(C.c_double), _I64, _I, _VP]),
    "trixi_batch_handle": (C.c_int, [_VP, _I64, C.POINTER(C.c_void_p)]),
    "trixi_batch_last_error": (C.c_int, [_VP, C.c_char_p, C.c_size_t]),
    "trixi_batch_tuning": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), _I64,
                                     C.POINTER(C.c_int64)]),
    "trixi_integrate": (C.c_int, [_VP, _DP, _DP, _I, C.POINTER(C.c_double), _I64, _VP]),
    "trixi_autotune": (C.c_int, [_VP, _VP, _VP]),
    "trixi_set_tile": (C.c_int, [_VP, _I, _I]),
    "trixi_tile": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                             C.POINTER(C.c_int), C.POINTER(C.c_double), _I64, C.POINTER(C.c_int64)]),
    "trixi_integrate_noalloc": (C.c_int, [_I, _I, _I, C.c_double, _VP, _VP, _VP, _I64, _I, _VP, _VP]),
    "trixi_calc_error_norms": (C.c_int, [_VP, _DP, _DP, _I, C.POINTER(C.c_double), _I64, _D,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double), _VP]),
    "trixi_set_glm_speed": (C.c_int, [_VP, _D]),
}

_lib = None


def library_path() -> Path:
    return _build.library_path()


def load(build_if_missing: bool = False):
    """Loads libtrixi_b200.so, raising if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


_diag = None


def load_diag():
    """Loads libtrixi_diag.so, the measurement diagnostics (FMA-peak probe,
    conversion check) that the benchmark and the tests use; not part of the
    rhs library."""
    global _diag
    if _diag is not None:
        return _diag
    path = _build.diag_library_path()
    if not path.exists():
        raise ImportError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(path))
    lib.trixi_diag_fma_peak.restype = C.c_int
    lib.trixi_diag_fma_peak.argtypes = [_I, _I, C.POINTER(C.c_double), _VP]
    lib.trixi_diag_convert.restype = C.c_int
    lib.trixi_diag_convert.argtypes = [_VP, _VP, _VP, _VP, _I64, _VP]
    _diag = lib
    return lib


def last_error(handle=None) -> str:
    buf = C.create_string_buffer(1024)
    load().trixi_last_error(handle, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, handle=None) -> None:
    if status != TRIXI_OK:
        raise TrixiError(status, last_error(handle))
