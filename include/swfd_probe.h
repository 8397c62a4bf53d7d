/*
 * swfd_probe.h -- measurement and test entry points of libswfd_probe.so.
 *
 * Not part of the product ABI (include/swfd.h) and with no counterpart in the
 * reference: the benchmark uses the FP64 throughput probe as the denominator
 * of the FP64-pipe roofline, and the tests use the others to check the
 * FP32-bulk form's reciprocal and conversions against IEEE arithmetic and
 * the persistent kernels' grid barrier's bounded wait.  The
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
/* Test entry point: two blocks of a cooperative launch at the persistent
 * kernels' grid barrier, the second absent when `absent` is set.  The wait
 * must end after wait_ms (0 < wait_ms <= 2000) with the timeout bit (64) in
 * *err_bits, without a fault; *passed counts the blocks that passed it. */
swfd_status swfd_probe_barrier_timeout(int32_t device, int32_t absent, double wait_ms,
                                       int32_t* err_bits, int32_t* passed);

/* Two blocks of a cooperative launch at one grid reduction of the
 * persistent 1D solve (per-block words polled by every block; block b posts
 * the value b + 1, block 0 a failed-positivity flag), the second absent
 * when `absent` is set.  The polls must end after wait_ms (0 < wait_ms <=
 * 2000) with the timeout bit (64) in *err_bits, without a fault; *passed
 * counts the blocks whose reduction completed and am_max[b], bad_flag[b]
 * (two entries each) hold what block b received. */
/* Host only (no device): the ranges of block b of the persistent 1D solve
 * for nx cells and `cells` cells per block, from the kernel's own layout
 * function: out[0..9] = a0, a1, nown (owned cells [a0, a1)), f0, f1, nf
 * (interface-flux cells [f0, f1]), s0, ns (split cells [s0, s0 + ns)), nhl,
 * nhr (halo cells below a0 and from a1 up); offsets 0..nx+5, cell i at
 * i + 2. */
swfd_status swfd_probe_solve1d_layout(int32_t nx, int32_t cells, int32_t b, int32_t* out);
swfd_status swfd_probe_reduce_timeout(int32_t device, int32_t absent, double wait_ms,
                                      int32_t* err_bits, int32_t* passed, double* am_max,
                                      int32_t* bad_flag);

#ifdef __cplusplus
}
#endif
#endif /* SWFD_PROBE_H */
