// swfd_probe.cu -- FP64 pipe throughput probe.  The FP64 path of this library
// is bounded by the FP64 pipe, whose peak is not a published constant of
// this part; this kernel measures it (independent DFMA chains, 8 per thread).
// Also test entry points: the FP32-bulk reciprocal and conversions, and the
// persistent kernels' bounded grid barrier and grid reduction.
#include <string.h>

#include "swfd_internal.h"
#include "swfd_device.cuh"
#include "swfd_gridsync.cuh"

namespace {

__global__ void k_dfma_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int k = 0; k < iters; ++k) {
    x0 = __fma_rn(x0, a, b); x1 = __fma_rn(x1, a, b); x2 = __fma_rn(x2, a, b);
    x3 = __fma_rn(x3, a, b); x4 = __fma_rn(x4, a, b); x5 = __fma_rn(x5, a, b);
    x6 = __fma_rn(x6, a, b); x7 = __fma_rn(x7, a, b);
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}

__global__ void k_rcp_bulk(const double* __restrict__ x, double* __restrict__ out, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    out[k] = swfd::rcp_bulk(x[k]);
}

__global__ void k_convert(const double* __restrict__ x, float* __restrict__ f,
                          double* __restrict__ d, int64_t n) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const float v = swfd::d2f(x[k]);
    f[k] = v;
    d[k] = swfd::f2d(v);
  }
}
// two blocks at one grid barrier; with `absent` the second block returns
// without arriving, so the first one's wait runs out
__global__ void k_barrier_probe(unsigned* cnt, int* err, int* passed, int absent,
                                unsigned long long wait_ns) {
  if (absent && blockIdx.x == 1) return;
  const bool ok = swfd::grid_barrier(cnt, 1, err, wait_ns);
  if (threadIdx.x == 0 && ok) atomicAdd(passed, 1);
}
// two blocks at one reduction of the persistent 1D solve (block b posts the
// value b + 1, block 0 the flag); with `absent` the second block returns
// without posting, so the first one's polls run out
__global__ void k_reduce_probe(unsigned long long* red, int* err, int* passed, double* am_out,
                               int* bad_out, int absent, unsigned long long wait_ns) {
  __shared__ double am;
  __shared__ int bad;
  if (absent && blockIdx.x == 1) return;
  const double v = threadIdx.x == 0 ? (double)(blockIdx.x + 1) : 0.0;
  const int f = blockIdx.x == 0 && threadIdx.x == 0;
  const bool ok = swfd::grid_reduce_2w(red, 1, err, wait_ns,
                                       (unsigned long long)__double_as_longlong(v), f, &am, &bad);
  if (threadIdx.x == 0 && ok) {
    atomicAdd(passed, 1);
    am_out[blockIdx.x] = am;
    bad_out[blockIdx.x] = bad;
  }
}
}  // namespace

// The persistent 1D solve's grid reduction with one block absent (or,
// absent = 0, both present): the polls of the other block must end after
// wait_ms with ERR_BIT_TIMEOUT in *err_bits and the context stay usable;
// *passed counts the blocks whose reduction completed, am_max[b] and
// bad_flag[b] (two each) what block b received.
extern "C" swfd_status swfd_probe_reduce_timeout(int32_t device, int32_t absent, double wait_ms,
                                                 int32_t* err_bits, int32_t* passed,
                                                 double* am_max, int32_t* bad_flag) {
  if (!err_bits || !passed || !am_max || !bad_flag || !(wait_ms > 0.0) || wait_ms > 2000.0)
    return SWFD_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return SWFD_ERR_CUDA;
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) return SWFD_ERR_UNSUPPORTED;
  // three sets of two words, SWFD_SOLVE1D_WSTRIDE apart; then err, passed,
  // the two blocks' results
  const size_t nred = 3 * 2 * SWFD_SOLVE1D_WSTRIDE;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, (nred + 8) * sizeof(unsigned long long)) != cudaSuccess) return SWFD_ERR_OOM;
  cudaError_t e = cudaMemset(d, 0xff, nred * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(d + nred, 0, 8 * sizeof(unsigned long long));
  unsigned long long* red = d;
  int* err = (int*)(d + nred);
  int* pass = err + 1;
  double* am = (double*)(d + nred + 2);
  int* bad = (int*)(d + nred + 4);
  int ab = absent ? 1 : 0;
  unsigned long long ns = (unsigned long long)(wait_ms * 1e6);
  void* args[] = {&red, &err, &pass, &am, &bad, &ab, &ns};
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((const void*)k_reduce_probe, dim3(2), dim3(64), args, 0,
                                    nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  unsigned long long h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpy(h, d + nred, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  int hi[4];
  double hd[2];
  memcpy(hi, h, sizeof(hi));
  memcpy(hd, h + 2, sizeof(hd));
  int hb[2];
  memcpy(hb, h + 4, sizeof(hb));
  *err_bits = hi[0];
  *passed = hi[1];
  am_max[0] = hd[0], am_max[1] = hd[1];
  bad_flag[0] = hb[0], bad_flag[1] = hb[1];
  return e == cudaSuccess ? SWFD_OK : SWFD_ERR_CUDA;
}

// The ranges of block b of the persistent 1D solve for nx cells (LI = nx + 6
// with the ghosts) and `cells` per block, on the host: the kernel's own
// layout function, for the in-bounds test of every shape
extern "C" swfd_status swfd_probe_solve1d_layout(int32_t nx, int32_t cells, int32_t b,
                                                 int32_t* out) {
  if (!out || nx < 1 || cells < 1 || b < 0 || b * (int64_t)cells >= (int64_t)nx + 6)
    return SWFD_ERR_INVALID;
  const swfd::Solve1dLayout L = swfd::solve1d_layout(b, cells, nx + 6, nx);
  const int32_t v[10] = {L.a0, L.a1, L.nown, L.f0, L.f1, L.nf, L.s0, L.ns, L.nhl, L.nhr};
  memcpy(out, v, sizeof(v));
  return SWFD_OK;
}

// The persistent kernels' grid barrier with one block absent (or, absent =
// 0, all present): the wait of the other block must end after wait_ms with
// ERR_BIT_TIMEOUT in *err_bits and the context stay usable; *passed counts
// the blocks that passed the barrier.
extern "C" swfd_status swfd_probe_barrier_timeout(int32_t device, int32_t absent, double wait_ms,
                                                  int32_t* err_bits, int32_t* passed) {
  if (!err_bits || !passed || !(wait_ms > 0.0) || wait_ms > 2000.0) return SWFD_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return SWFD_ERR_CUDA;
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) return SWFD_ERR_UNSUPPORTED;
  int* d = nullptr;
  if (cudaMalloc(&d, 4 * sizeof(int)) != cudaSuccess) return SWFD_ERR_OOM;
  cudaError_t e = cudaMemset(d, 0, 4 * sizeof(int));
  unsigned* cnt = (unsigned*)d;
  int* err = d + 1;
  int* pass = d + 2;
  int ab = absent ? 1 : 0;
  unsigned long long ns = (unsigned long long)(wait_ms * 1e6);
  void* args[] = {&cnt, &err, &pass, &ab, &ns};
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(2), dim3(32), args, 0,
                                    nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int h[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, 4 * sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  *err_bits = h[1];
  *passed = h[2];
  return e == cudaSuccess ? SWFD_OK : SWFD_ERR_CUDA;
}

// the integer-pipe binary64 -> binary32 -> binary64 conversions of the
// FP32-bulk kernels on host values, for their bit-exactness test
extern "C" swfd_status swfd_probe_convert(int32_t device, const double* x, int64_t n,
                                          float* out_f, double* out_d) {
  if (!x || !out_f || !out_d || n < 0 || n > (int64_t)1 << 26) return SWFD_ERR_INVALID;
  if (n == 0) return SWFD_OK;
  if (cudaSetDevice(device) != cudaSuccess) return SWFD_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, 2 * n * sizeof(double) + n * sizeof(float)) != cudaSuccess) return SWFD_ERR_OOM;
  float* f = (float*)(d + 2 * n);
  cudaError_t e = cudaMemcpy(d, x, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_convert<<<256, 256>>>(d, f, d + n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out_f, f, n * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(out_d, d + n, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? SWFD_OK : SWFD_ERR_CUDA;
}

// the FP32-bulk reciprocal on host values, for its error-bound test
extern "C" swfd_status swfd_probe_rcp_bulk(int32_t device, const double* x, int64_t n,
                                           double* out) {
  if (!x || !out || n < 0 || n > (int64_t)1 << 26) return SWFD_ERR_INVALID;
  if (n == 0) return SWFD_OK;
  if (cudaSetDevice(device) != cudaSuccess) return SWFD_ERR_CUDA;
  double* d = nullptr;
  if (cudaMalloc(&d, 2 * n * sizeof(double)) != cudaSuccess) return SWFD_ERR_OOM;
  cudaError_t e = cudaMemcpy(d, x, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_rcp_bulk<<<256, 256>>>(d, d + n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + n, n * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? SWFD_OK : SWFD_ERR_CUDA;
}

extern "C" swfd_status swfd_probe_fp64_peak(int32_t device, double* gflops) {
  if (!gflops) return SWFD_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return SWFD_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* out = nullptr;
  if (cudaMalloc(&out, 1 << 20) != cudaSuccess) return SWFD_ERR_OOM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8, iters = 4096;
  k_dfma_probe<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_dfma_probe<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return SWFD_ERR_CUDA;
  *gflops = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3) / 1e9;
  return SWFD_OK;
}
