// Fused DGSEM kernels for 2D ideal GLM-MHD on non-periodic meshes, compute type double.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_2d_f64_mhd_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  if (eq != EQ_MHD) return cudaErrorNotSupported;
  return launch_dim_mhd<2, double, 1>(N, vol, vflux, h, s);
}
}  // namespace trixi
