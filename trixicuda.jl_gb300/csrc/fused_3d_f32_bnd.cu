// Fused DGSEM kernels for 3D, compute type float: non-periodic meshes and/or source terms.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_3d_f32_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  return launch_dim<3, float, 1>(N, eq, vol, vflux, h, s);
}
}  // namespace trixi
