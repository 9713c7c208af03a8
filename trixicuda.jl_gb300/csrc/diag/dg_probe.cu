// dg_probe.cu -- measurement diagnostics of libtrixi_diag.so (not part of
// libtrixi_b200.so): the CUDA-core FMA throughput probe (FP64 / FP32) and the
// elementwise integer-pipe conversions of the mixed-precision kernels.
//
// The roofline of the FP64 flux-differencing kernels is the FP64 pipe, whose
// peak on GB300 is not published with the HBM and tensor peaks; this kernel
// measures it: every thread runs 8 independent FMA chains, enough blocks are
// launched to fill every SM, and the kernel is timed with CUDA events.
#include <cuda_runtime.h>

#include <cstdint>

#include "trixi_diag.h"
#include "../dg_convert.cuh"

namespace {

template <typename R>
__global__ void fma_chains(R *out, int iters, R a, R b) {
  R x0 = R(threadIdx.x) * R(1e-3), x1 = x0 + R(1), x2 = x0 + R(2), x3 = x0 + R(3);
  R x4 = x0 + R(4), x5 = x0 + R(5), x6 = x0 + R(6), x7 = x0 + R(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  const R s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == R(-12345.678)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keep the chains live
}

template <typename R>
int run(int iters, double *flops_per_s, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256, grid = sms * 8;
  R *out = nullptr;
  if (cudaMalloc(&out, sizeof(R) * (size_t)grid * block) != cudaSuccess) return TRIXI_DIAG_ERR_OUT_OF_MEMORY;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<R><<<grid, block, 0, s>>>(out, iters / 8 + 1, R(0.999999), R(1e-7));  // warm-up
  cudaEventRecord(e0, s);
  fma_chains<R><<<grid, block, 0, s>>>(out, iters, R(0.999999), R(1e-7));
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess || ms <= 0.f) return TRIXI_DIAG_ERR_CUDA;
  const double fmas = (double)grid * block * (double)iters * 16.0 * 8.0;
  *flops_per_s = 2.0 * fmas / (ms * 1e-3);
  return TRIXI_DIAG_OK;
}

}  // namespace

extern "C" int trixi_diag_fma_peak(int precision, int iters, double *flops_per_s, void *stream) {
  if (!flops_per_s || iters <= 0) return TRIXI_DIAG_ERR_INVALID_ARGUMENT;
  if (precision == TRIXI_DIAG_FP64) return run<double>(iters, flops_per_s, (cudaStream_t)stream);
  return run<float>(iters, flops_per_s, (cudaStream_t)stream);
}

namespace {
__global__ void convert_kernel(const double *in_d, float *out_f, const float *in_f, double *out_d, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out_f[i] = trixi::d2f_rn(in_d[i]);
  out_d[i] = trixi::f2d_exact(in_f[i]);
}
}  // namespace

extern "C" int trixi_diag_convert(const double *in_d, float *out_f, const float *in_f, double *out_d, int64_t n,
                                   void *stream) {
  if (n < 0 || (n > 0 && (!in_d || !out_f || !in_f || !out_d))) return TRIXI_DIAG_ERR_INVALID_ARGUMENT;
  if (n == 0) return TRIXI_DIAG_OK;
  convert_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(in_d, out_f, in_f, out_d, n);
  return cudaGetLastError() == cudaSuccess ? TRIXI_DIAG_OK : TRIXI_DIAG_ERR_CUDA;
}
