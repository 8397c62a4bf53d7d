// swfd_control.h -- launchers of the device-side control kernels.
#pragma once

#include "swfd_internal.h"

namespace swfd {

cudaError_t launch_restart_init(cudaGraphConditionalHandle hw, DevScalars* d, cudaStream_t s);
cudaError_t launch_restart_begin(DevScalars* d, cudaStream_t s);
cudaError_t launch_restart_end(cudaGraphConditionalHandle hw, DevScalars* d, cudaStream_t s);
cudaError_t launch_restart_commit(const Params& p, const double* src, double* dst,
                                  const DevScalars* d, cudaStream_t s);
cudaError_t launch_cond_density(cudaGraphConditionalHandle h, DevScalars* d, cudaStream_t s);
cudaError_t launch_count_density(DevScalars* d, cudaStream_t s);
cudaError_t launch_sweep_begin(cudaGraphConditionalHandle h, const Params& p, DevScalars* d,
                               int check_pubar, int swp_num, cudaStream_t s);
cudaError_t launch_q_begin(const Params& p, DevScalars* d, cudaStream_t s);
cudaError_t launch_q_end(cudaGraphConditionalHandle h, DevScalars* d, int swp_num, int stop_on_fail,
                         cudaStream_t s);
cudaError_t launch_run_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop,
                            cudaStream_t s);
cudaError_t launch_time_advance_cond(cudaGraphConditionalHandle h, DevScalars* d, double t_loop,
                                     cudaStream_t s);

}  // namespace swfd
