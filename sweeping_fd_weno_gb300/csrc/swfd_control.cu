// swfd_control.cu -- single-thread kernels that take the decisions the
// reference takes on the host between its loops, so that a step (and a whole
// solve) runs as one CUDA graph: they update the statistics counters and set
// the values of the graph's conditional nodes (IF / WHILE).
#include "swfd_control.h"

namespace swfd {

__device__ __forceinline__ double decode_key(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// restart RK (ex2_sedov_1d/main.f90:330-374).  After the step's first
// wenofd and dt: alphatemp = alphamax (:337), enter the loop.
__global__ void k_restart_init(cudaGraphConditionalHandle hw, DevScalars* d) {
  d->alphatemp = d->alphamax;
  d->restarts = 0;
  set_cond(hw, &d->cond, 1u);
}

// label 110 (:339-346): a restart halves dt and restores alphamax; stage 1
// reads u0 itself, so `u = u0` is implicit.  postag starts at 0.
__global__ void k_restart_begin(DevScalars* d) {
  if (d->restarts > 0) {
    d->dt = d->dt / 2.;
    d->alphamax = d->alphatemp;
  }
  d->postag = 0;
}

// `if (postag == 1) goto 110` (:350, :360, :370), bounded by SWFD_RESTART_LIMIT
__global__ void k_restart_end(cudaGraphConditionalHandle hw, DevScalars* d) {
  unsigned go = 0;
  if (d->postag) {
    if (d->restarts >= SWFD_RESTART_LIMIT) {
      d->error |= ERR_BIT_RESTART;
    } else {
      d->restarts++;
      d->restart_total++;
      go = 1;
    }
  }
  set_cond(hw, &d->cond, go);
}

// the accepted stage-3 state becomes u (whole planes, ghosts included),
// unless the step gave up
__global__ void k_restart_commit(const double* __restrict__ src, double* __restrict__ dst,
                                 int64_t n, const DevScalars* d) {
  if (d->error & ERR_BIT_RESTART) return;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    dst[k] = src[k];
}

// IF rho_min < 1d-12 (ex3_vortex_accuracy_2d/main.f90:1155-1156); den_count (:1187)
__global__ void k_cond_density(cudaGraphConditionalHandle h, DevScalars* d) {
  bool go = decode_key(d->rho_min_key) < 1e-12;
  if (go) d->den_count++;
  set_cond(h, &d->cond, go ? 1u : 0u);
}

// 1D: the density sweep always runs (ex2_sedov_1d/main.f90:774)
__global__ void k_count_density(DevScalars* d) { d->den_count++; }

// sweep_lim set-up after u_bar (ex3_vortex_accuracy_2d/main.f90:928-930;
// ex4's P(u_bar) <= 0 stop, ex4_sedov_2d/main.f90:1447-1454)
__global__ void k_sweep_begin(cudaGraphConditionalHandle h, Params p, DevScalars* d,
                              int check_pubar, int swp_num) {
  if (check_pubar) {
    const double* ub = d->ubar;
    if (p.gamma1 * (ub[3] - 0.5 * (ub[1] * ub[1] + ub[2] * ub[2]) / ub[0]) <= 0.) {
      d->error |= ERR_BIT_PUBAR;
      set_cond(h, &d->cond, 0u);
      return;
    }
  }
  long long k = d->sweep_count++;
  if (k < d->track_cap) {
    d->tracks[k] = 0;
    d->tracks[d->track_cap + k] = 0;
    d->tracks[2 * d->track_cap + k] = 0;
  }
  d->t_pos = 0;
  d->t_neg = 0;
  d->q = 0;
  set_cond(h, &d->cond, swp_num >= 1 ? 1u : 0u);
}

// start of sweep iteration q: odd q ordering I, even q ordering II (:933)
__global__ void k_q_begin(Params p, DevScalars* d) {
  int q = ++d->q;
  d->ordering = p.g.ndim == 1 ? 0 : ((q & 1) ? 1 : 2);
}

// end of sweep iteration q: pre_count, exit test and tracks (:1116-1129)
__global__ void k_q_end(cudaGraphConditionalHandle h, DevScalars* d, int swp_num, int stop_on_fail) {
  d->pre_count++;
  if (d->error & ERR_BIT_CHECK) {  // ex6 stopped inside the passes
    set_cond(h, &d->cond, 0u);
    return;
  }
  if (d->bad_count == 0) {
    long long k = d->sweep_count - 1;
    if (k >= 0 && k < d->track_cap) {
      d->tracks[k] = d->q;
      d->tracks[d->track_cap + k] = (int)d->t_neg;
      d->tracks[2 * d->track_cap + k] = (int)d->t_pos;
    }
    set_cond(h, &d->cond, 0u);
    return;
  }
  if (d->q >= swp_num) {
    d->fail_count++;
    if (stop_on_fail) d->error |= ERR_BIT_NOCONV;
    set_cond(h, &d->cond, 0u);
    return;
  }
  set_cond(h, &d->cond, 1u);
}

// DO WHILE (time <= time_terminal - 1d-10) (ex3_vortex_accuracy_2d/main.f90:51),
// bounded by the launch's step limit and stopped by an error
__global__ void k_run_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop) {
  bool go = (d->time <= t_loop) && (d->steps < d->steps_limit) && (d->error == 0);
  set_cond(h, &d->cond, go ? 1u : 0u);
}

// time = time + dt (:53), then the loop test
__global__ void k_time_advance_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop) {
  d->time = d->time + d->dt;
  d->steps++;
  bool go = (d->time <= t_loop) && (d->steps < d->steps_limit) && (d->error == 0);
  set_cond(h, &d->cond, go ? 1u : 0u);
}

cudaError_t launch_restart_init(cudaGraphConditionalHandle hw, DevScalars* d, cudaStream_t s) {
  k_restart_init<<<1, 1, 0, s>>>(hw, d);
  return cudaGetLastError();
}
cudaError_t launch_restart_begin(DevScalars* d, cudaStream_t s) {
  k_restart_begin<<<1, 1, 0, s>>>(d);
  return cudaGetLastError();
}
cudaError_t launch_restart_end(cudaGraphConditionalHandle hw, DevScalars* d, cudaStream_t s) {
  k_restart_end<<<1, 1, 0, s>>>(hw, d);
  return cudaGetLastError();
}
cudaError_t launch_restart_commit(const Params& p, const double* src, double* dst,
                                  const DevScalars* d, cudaStream_t s) {
  const int64_t n = (int64_t)p.g.nc * p.g.plane;
  const unsigned gb = (unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
  k_restart_commit<<<gb, 256, 0, s>>>(src, dst, n, d);
  return cudaGetLastError();
}
cudaError_t launch_cond_density(cudaGraphConditionalHandle h, DevScalars* d, cudaStream_t s) {
  k_cond_density<<<1, 1, 0, s>>>(h, d);
  return cudaGetLastError();
}
cudaError_t launch_count_density(DevScalars* d, cudaStream_t s) {
  k_count_density<<<1, 1, 0, s>>>(d);
  return cudaGetLastError();
}
cudaError_t launch_sweep_begin(cudaGraphConditionalHandle h, const Params& p, DevScalars* d,
                               int check_pubar, int swp_num, cudaStream_t s) {
  k_sweep_begin<<<1, 1, 0, s>>>(h, p, d, check_pubar, swp_num);
  return cudaGetLastError();
}
cudaError_t launch_q_begin(const Params& p, DevScalars* d, cudaStream_t s) {
  k_q_begin<<<1, 1, 0, s>>>(p, d);
  return cudaGetLastError();
}
cudaError_t launch_q_end(cudaGraphConditionalHandle h, DevScalars* d, int swp_num, int stop_on_fail,
                         cudaStream_t s) {
  k_q_end<<<1, 1, 0, s>>>(h, d, swp_num, stop_on_fail);
  return cudaGetLastError();
}
cudaError_t launch_run_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop,
                            cudaStream_t s) {
  k_run_cond<<<1, 1, 0, s>>>(h, d, t_loop);
  return cudaGetLastError();
}
cudaError_t launch_time_advance_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop,
                                     cudaStream_t s) {
  k_time_advance_cond<<<1, 1, 0, s>>>(h, d, t_loop);
  return cudaGetLastError();
}

}  // namespace swfd
