// Fused DGSEM kernels for 3D ideal GLM-MHD on non-periodic meshes, compute type float.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_3d_f32_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  if (eq != EQ_MHD) return cudaErrorNotSupported;
  return launch_dim_mhd<3, float, 1>(N, vol, vflux, h, s);
}
}  // namespace trixi
