/*
 * trixi_diag.h -- C ABI of libtrixi_diag.so, the measurement diagnostics that
 * the benchmark and the tests load beside libtrixi_b200.so.  They are not part
 * of the rhs library and have no counterpart in the reference.
 */
#ifndef TRIXI_DIAG_H
#define TRIXI_DIAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { TRIXI_DIAG_OK = 0, TRIXI_DIAG_ERR_INVALID_ARGUMENT = 1, TRIXI_DIAG_ERR_CUDA = 3,
       TRIXI_DIAG_ERR_OUT_OF_MEMORY = 6 };
enum { TRIXI_DIAG_FP64 = 0, TRIXI_DIAG_FP32 = 1 };

/* CUDA-core FMA throughput (FLOP/s, 2 per FMA) of the current device in FP64
 * or FP32: every thread runs 8 independent FMA chains on 8 blocks per SM,
 * timed with CUDA events.  Synchronizes the stream. */
int trixi_diag_fma_peak(int precision, int iters, double *flops_per_s, void *stream);

/* The mixed-precision kernels' integer-pipe conversions (double -> float,
 * round to nearest even; float -> double, exact) applied elementwise to
 * device arrays of length n, for bit-for-bit comparison with the hardware
 * conversions. */
int trixi_diag_convert(const double *in_d, float *out_f, const float *in_f, double *out_d, int64_t n,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif /* TRIXI_DIAG_H */
