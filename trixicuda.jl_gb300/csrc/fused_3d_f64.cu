// Fused DGSEM kernels for 3D, compute type double: periodic meshes without source terms.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_3d_f64(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  return launch_dim<3, double, 0>(N, eq, vol, vflux, h, s);
}
}  // namespace trixi
