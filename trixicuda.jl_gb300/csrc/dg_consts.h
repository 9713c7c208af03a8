// dg_consts.h -- enumerations shared by host code and kernels.  The numeric
// values equal the public trixi_* enums of include/trixi_b200.h.
#pragma once
#include <cstdint>

namespace trixi {

constexpr int EQ_ADV = 0;    // TRIXI_EQ_LINEAR_ADVECTION
constexpr int EQ_EULER = 1;  // TRIXI_EQ_COMPRESSIBLE_EULER
constexpr int EQ_MHD = 2;    // TRIXI_EQ_IDEAL_GLM_MHD

constexpr int FLUX_LLF = 0;        // TRIXI_FLUX_LAX_FRIEDRICHS
constexpr int FLUX_RANOCHA = 1;    // TRIXI_FLUX_RANOCHA
constexpr int FLUX_CENTRAL = 2;    // TRIXI_FLUX_CENTRAL
constexpr int FLUX_LLF_NAIVE = 3;  // TRIXI_FLUX_LAX_FRIEDRICHS_NAIVE
constexpr int FLUX_HG = 4;         // TRIXI_FLUX_HINDENLANG_GASSNER
constexpr int FLUX_SHIMA = 5;      // TRIXI_FLUX_SHIMA_ETAL
constexpr int FLUX_HLL = 6;        // TRIXI_FLUX_HLL
constexpr int FLUX_HLLE = 7;       // TRIXI_FLUX_HLLE

constexpr int NONCONS_NONE = 0;    // TRIXI_NONCONSERVATIVE_NONE
constexpr int NONCONS_POWELL = 1;  // TRIXI_NONCONSERVATIVE_POWELL

constexpr int VOL_WEAK = 0;  // TRIXI_VOLUME_WEAK_FORM
constexpr int VOL_FD = 1;    // TRIXI_VOLUME_FLUX_DIFFERENCING
constexpr int VOL_SC = 2;    // TRIXI_VOLUME_SHOCK_CAPTURING_HG

constexpr int MODE_VOLUME = 0;  // du = volume integral only (stage API)
constexpr int MODE_RHS = 1;     // du = full rhs
constexpr int MODE_RK = 2;      // k = a k + dt rhs; u_out = u_in + b k

// face-table entry of a face on a non-periodic domain boundary (neighbours
// are >= 0, mortar slots -(slot+1))
constexpr int32_t FACE_BOUNDARY = INT32_MIN;

}  // namespace trixi
