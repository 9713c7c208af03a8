// Fused DGSEM kernels for 1D, compute type double: non-periodic meshes and/or source terms.
#include "dg_launch.cuh"

namespace trixi {
cudaError_t launch_fused_1d_f64_bnd(int N, int eq, int vol, int vflux, const FusedHost &h, cudaStream_t s) {
  return launch_dim<1, double, 1>(N, eq, vol, vflux, h, s);
}
}  // namespace trixi
