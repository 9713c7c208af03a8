"""trixicuda -- host-side mirror of TrixiCUDA.jl's public API on top of the
GB300 (sm_103a) C-ABI library libtrixi_b200.so.

Names follow the reference (src/TrixiCUDA.jl:70-73 exports DGSEMGPU,
SemidiscretizationHyperbolicGPU, semidiscretizeGPU, LobattoLegendreBasisGPU)
plus the Trixi.jl names its users pass in (TreeMesh, equations, fluxes,
volume integrals, IndicatorHennemannGassner) and the stage functions its
tests call (`cuda_*`, `rhs_gpu`).  Julia's trailing `!` is dropped.
"""
from . import _lib
from .equations import (
    CompressibleEulerEquations1D,
    CompressibleEulerEquations2D,
    CompressibleEulerEquations3D,
    IdealGlmMhdEquations1D,
    IdealGlmMhdEquations2D,
    IdealGlmMhdEquations3D,
    LinearScalarAdvectionEquation1D,
    LinearScalarAdvectionEquation2D,
    LinearScalarAdvectionEquation3D,
    flux,
    flux_central,
    flux_hindenlang_gassner,
    flux_hll,
    flux_hlle,
    flux_lax_friedrichs,
    flux_lax_friedrichs_naive,
    flux_nonconservative_powell,
    flux_ranocha,
    flux_shima_etal,
    initial_condition_constant,
    initial_condition_convergence_test,
    initial_condition_eoc_test_coupled_euler_gravity,
    initial_condition_fourier_advection,
    initial_condition_fourier_euler,
    initial_condition_weak_blast_wave,
    BoundaryConditionDirichlet,
    boundary_condition_periodic,
    source_terms_convergence_test,
    source_terms_eoc_test_euler,
)
from .mesh import TreeMesh
from .semidiscretization import (
    ODEProblem,
    SemidiscretizationHyperbolicGPU,
    autotune,
    set_tile,
    set_glm_speed,
    calc_error_norms,
    compute_coefficients_gpu,
    integrate,
    max_dt,
    cuda_boundary_flux,
    cuda_indicator,
    cuda_interface_flux,
    cuda_jacobian,
    cuda_mortar_flux,
    cuda_prolong2boundaries,
    cuda_prolong2interfaces,
    cuda_prolong2mortars,
    cuda_sources,
    cuda_surface_integral,
    cuda_volume_integral,
    rhs_gpu,
    rk_stage,
    rk_steps,
    rk_steps_host,
    semidiscretizeGPU,
    synchronize,
    tile,
    wrap_array,
)
from .solver import (
    DGSEMGPU,
    IndicatorHennemannGassner,
    LobattoLegendreBasisGPU,
    VolumeIntegralFluxDifferencing,
    VolumeIntegralShockCapturingHG,
    VolumeIntegralWeakForm,
    density_pressure,
    pressure,
)
from .time_integration import CarpenterKennedy2N54, solve

TrixiError = _lib.TrixiError

__version__ = "0.1.0"
