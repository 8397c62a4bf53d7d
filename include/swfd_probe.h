/*
 * swfd_probe.h -- measurement and test entry points of libswfd_probe.so.
 *
 * Not part of the product ABI (include/swfd.h) and with no counterpart in the
 * reference: the benchmark uses the FP64 throughput probe as the denominator
 * of the FP64-pipe roofline, and the tests use the other two to check the
 * FP32-bulk form's reciprocal and conversions against IEEE arithmetic.  The
 * kernels run the same device functions as libswfd.so (swfd_device.cuh).
 */
#ifndef SWFD_PROBE_H
#define SWFD_PROBE_H

#include "swfd.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Measured FP64 FMA throughput of the device in GFLOP/s (2 flops per FMA):
 * the denominator of the FP64-pipe roofline of the FP64 path. */
swfd_status swfd_probe_fp64_peak(int32_t device, double* gflops);
/* The FP32-bulk form's reciprocal (the correctly rounded quotient 1/x of the
 * library's software binary64 division) applied to n host values on the
 * device, for its error test. */
swfd_status swfd_probe_rcp_bulk(int32_t device, const double* x, int64_t n, double* out);
/* Test entry point: the FP32-bulk kernels' binary64 -> binary32 conversion
 * (out_f) and its binary32 -> binary64 widening (out_d), both on the integer
 * pipes, for n host values; they must equal the hardware conversions. */
swfd_status swfd_probe_convert(int32_t device, const double* x, int64_t n, float* out_f,
                               double* out_d);

#ifdef __cplusplus
}
#endif
#endif /* SWFD_PROBE_H */
