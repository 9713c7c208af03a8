// Fused DGSEM kernels for 1D, compute type float: periodic meshes without source terms.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_1d_f32(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  return launch_dim<1, float, 0>(N, eq, vol, vflux, h, s);
}
}  // namespace trixi
