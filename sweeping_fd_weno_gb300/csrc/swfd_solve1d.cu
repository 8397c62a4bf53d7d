// swfd_solve1d.cu -- the 1D point-energy solve (ex2_sedov_1d/main.f90: the
// time loop :38-53 over the SSP-RK3 step rk3 :287-328) as one persistent kernel.
//
// An 800-cell stage is a few microseconds of dependent FP64 chains; as four
// graph kernels per stage (findalpha, splitting, fluxes, RK stage) its time
// is the kernels' launch and drain latencies.  Here a cooperative grid of
// one block per SM runs the whole time loop.  Each block owns a contiguous
// range of cells and, per stage, computes in shared memory the split fluxes
// of its range plus a three-cell halo, the interface fluxes of its range
// plus one, the RK stage of its own cells, their positivity and their
// findalpha term for the next stage; one grid barrier per stage then makes
// the stage's state, the maximum alpha and the positivity flag visible to
// every block.  A stage whose state fails checkpositivity ends the launch:
// the host runs sweep_lim on it and launches again at the next stage.
//
// Every value is computed by the separate kernels' code (swfd_1d.cuh).
#include "swfd_1d.cuh"
#include "swfd_gridsync.cuh"

namespace swfd {
namespace {

// a grid barrier gives up after 2 s of waiting (the slowest legitimate wait
// is one stage of the other blocks, microseconds)
constexpr unsigned long long S1_WAIT_NS = 2000000000ull;

// maximum over the block (values >= 0) and the OR of the flags, in every thread
__device__ __forceinline__ void s1_block_reduce(double& v, int& f) {
  __shared__ double wm[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wm[w] = v;
  f = __syncthreads_or(f);
  v = 0.0;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) v = fmax(v, wm[k]);
  __syncthreads();  // wm is rewritten by the next call
}

// an interface's eigenvectors in shared memory (S1_EIG planes of FW doubles)
constexpr int S1_EIG = 15;
__device__ __forceinline__ void s1_eig_store(const Eigen1D<double>& E, double* s, int FW, int j) {
  const double v[6] = {E.vxm, E.qm, E.r10, E.r12, E.r20, E.r22};
#pragma unroll
  for (int k = 0; k < 6; ++k) s[k * FW + j] = v[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) s[(6 + k) * FW + j] = E.L[k / 3][k % 3];
}
__device__ __forceinline__ void s1_eig_load(Eigen1D<double>& E, const double* s, int FW, int j) {
  E.vxm = s[j], E.qm = s[FW + j], E.r10 = s[2 * FW + j], E.r12 = s[3 * FW + j];
  E.r20 = s[4 * FW + j], E.r22 = s[5 * FW + j];
#pragma unroll
  for (int k = 0; k < 9; ++k) E.L[k / 3][k % 3] = s[(6 + k) * FW + j];
}

// the grid's maximum alpha and positivity flag from the blocks' parts
__device__ __forceinline__ void s1_grid_reduce(const Solve1dPart* parts, double& am, int& bad) {
  __shared__ double sa;
  __shared__ int sb;
  if (threadIdx.x < 32) {
    double v = 0.0;
    int f = 0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += 32) {
      v = fmax(v, parts[k].a);
      f |= parts[k].bad;
    }
    for (int o = 16; o > 0; o >>= 1) {
      v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
      f |= __shfl_xor_sync(0xffffffffu, f, o);
    }
    if (threadIdx.x == 0) sa = v, sb = f;
  }
  __syncthreads();
  am = sa;
  bad = sb;
  __syncthreads();  // sa, sb are rewritten by the next call
}

// The state buffers: st[0] = X (the step's start, u0, written back by stage
// 3), st[1] = Y, st[2] = Z; stage k reads st[k-1] and writes st[k % 3]
// (the rotation of the separate kernels' step).  The buffers change during
// the launch, so they are read with coherent loads.
__global__ void __launch_bounds__(SWFD_SOLVE1D_MAX_BLOCK)
    k_solve1d(Params p, Solve1dArgs a, DevScalars* dsc, double t_loop) {
  extern __shared__ double sm[];
  const Geom& g = p.g;
  const int n = g.nx, LI = g.LI;
  const int64_t P = g.plane;
  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  // owned cells [a0, a1) (offsets: cell i at i + 2), interface-flux cells
  // [f0, f1] within 2..n+3 (the reference's m = 0..n+1), split and state
  // cells [f0 - 2, f1 + 2]
  const int a0 = b * a.cells, a1 = min(LI, a0 + a.cells);
  const int f0 = max(a0 - 1, 2), f1 = min(a1, n + 3);
  const int nf = f1 - f0 + 1, s0 = f0 - 2, ns = nf + 4;
  const int SW = a.cells + 6, FW = a.cells + 2;
  double* ssp = sm;            // split: fp 0..2, fn 3..5, 6 x SW
  double* sfl = ssp + 6 * SW;  // interface fluxes: hp 0..2, hn 3..5, 6 x FW
  double* sev = sfl + 6 * FW;  // eigenvectors of the flux cells, S1_EIG x FW
  double* snew = sev + S1_EIG * FW;  // the stage's new state of the owned cells, 3 x cells
  // the split runs on threads [0, ns), the eigenvectors on the warps after
  // them, threads [ev0, ev0 + nf)
  const int ev0 = (ns + 31) & ~31;
  const double* u0 = a.st[0];
  const bool sweeps = a.sweeps != 0;

  double time = dsc->time, dt = dsc->dt, am = 0.0, am_next = 0.0;
  long long steps = dsc->steps;
  const long long lim = dsc->steps_limit;
  int err = 0, pause = 0, par = 0;
  unsigned nbar = 0;
  bool have_alpha = false;
  int stage = a.resume;
  if (stage == 4) {  // the step whose stage-3 sweep the host ran: time = time + dt (:44)
    time = time + dt;
    ++steps;
    stage = 1;
  }
  for (;;) {
    // DO WHILE (time <= time_terminal - 1d-10), within the launch's step bound
    if (stage == 1 && !(time <= t_loop && steps < lim && err == 0)) break;
    const double* in = a.st[stage - 1];
    double* out = a.st[stage % 3];
    if (!have_alpha) {  // findalpha (:273-285) over the stage's input
      double v = 0.0;
      int f = 0;
      for (int q = a0 + tid; q < a1; q += blockDim.x)
        v = fmax(v, fmax(0.0, alpha1d(p, in[q], in[P + q], in[2 * P + q])));
      s1_block_reduce(v, f);
      if (tid == 0) a.parts[par * G + b] = Solve1dPart{v, 0, 0};
      if (!grid_barrier(a.bar, ++nbar, &dsc->error, S1_WAIT_NS)) return;
      int unused;
      s1_grid_reduce(a.parts + par * G, am, unused);
      par ^= 1;
    } else {
      am = am_next;
    }
    if (!isfinite(am) || !(am > 0.0)) err |= ERR_BIT_ALPHA;
    if (stage == 1) {  // dt = dx*cfl/alphamax (:293)
      dt = p.dt_num_x / am;
      if (!isfinite(dt)) err |= ERR_BIT_DT;
    }
    if (tid < ns) {  // fflux and the split (:82-85) of cells s0 .. s0 + ns - 1
      const int q = s0 + tid;
      double sp[3], sn[3];
      split1d<double>(p, in[q], in[P + q], in[2 * P + q], am, sp, sn);
      for (int c = 0; c < 3; ++c) ssp[c * SW + tid] = sp[c], ssp[(3 + c) * SW + tid] = sn[c];
    } else if (tid >= ev0 && tid < ev0 + nf) {  // eigenvectors at flux cell f0 + j (:103-133)
      const int j = tid - ev0, q = f0 + j;
      Eigen1D<double> E;
      eigen1d<double>(p.gamma1, in[q], in[P + q], in[2 * P + q], E);
      s1_eig_store(E, sev, FW, j);
    }
    __syncthreads();
    {  // interface fluxes (:88-157), eight lanes per flux cell f0 + j
      const int j = tid >> 3, sub = tid & 7;
      const int jc = j < nf ? j : max(nf - 1, 0);  // lanes past the range repeat the last cell
      Eigen1D<double> E;
      s1_eig_load(E, sev, FW, jc);
      const double v = recon1d<double, false>(
          p, E, sub, [&](int side, int c, int jj) { return ssp[(3 * side + c) * SW + jc + jj]; });
      const double r = back1d<double>(E, v, sub);
      if (!p.limiter) {
        if (j < nf && sub < 6) sfl[sub * FW + j] = r;
      } else {  // use_limiter 1 (:159-245): lanes 0 and 3 limit their side
        double w[3];
        int nd = 0, np = 0;
        const bool lim = limit1d_group<double>(
            p, r, sub, [&](int side, int c) { return ssp[(3 * side + c) * SW + jc + 2]; }, w, nd,
            np);
        if (j < nf && lim) {
          for (int c = 0; c < 3; ++c) sfl[(sub + c) * FW + j] = w[c];
          // a flux cell next to the range is also the neighbour block's:
          // the block that owns the cell counts its limitings
          if (f0 + j >= a0 && f0 + j < a1)
            count_limited((unsigned long long*)&dsc->den_count, nd, np);
        }
      }
    }
    __syncthreads();
    // scheme (:252-271) and the RK stage of the owned cells, four lanes per
    // cell (lane c < 3: component c)
    const int nown = a1 - a0;
    {
      const int cell = tid >> 2, c = tid & 3, q = a0 + cell;
      const int i = q - 2;
      if (cell < nown && c < 3) {
        double r = 0.0;
        if (i >= 1 && i <= n) {
          const int k = q - f0;
          r = rhs1d_value<double>(p, am, sfl[c * FW + k - 1], sfl[(3 + c) * FW + k],
                                  sfl[c * FW + k], sfl[(3 + c) * FW + k + 1]);
        }
        const double v = rk1d_value<double>(p, stage, dt, r, in[c * P + q], u0 + c * P + q);
        out[c * P + q] = v;
        snew[c * a.cells + cell] = v;
      }
    }
    __syncthreads();
    // checkpositivity (:376-392) of the owned interior cells on the first
    // warp, the next stage's findalpha terms on the warp after it
    double av = 0.0;
    int bad = 0;
    const int aw = (nown + 31) & ~31;
    if (tid < nown) {
      const int i = a0 + tid - 2;
      if (i >= 1 && i <= n)
        bad = pos1d_bad<double>(p, snew[tid], snew[a.cells + tid], snew[2 * a.cells + tid]);
    } else if (tid >= aw && tid < aw + nown) {
      const int t = tid - aw;
      av = fmax(0.0, alpha1d(p, snew[t], snew[a.cells + t], snew[2 * a.cells + t]));
    }
    s1_block_reduce(av, bad);
    if (tid == 0) {
      a.parts[par * G + b] = Solve1dPart{av, bad, 0};
      if (b == 0) dsc->rk_runs[stage]++;
    }
    if (!grid_barrier(a.bar, ++nbar, &dsc->error, S1_WAIT_NS)) return;
    int postag;
    s1_grid_reduce(a.parts + par * G, am_next, postag);
    par ^= 1;
    have_alpha = true;
    if (postag && sweeps) {  // sweep_lim runs on the host's launches
      pause = stage;
      break;
    }
    if (stage == 3) {  // time = time + dt (:44)
      time = time + dt;
      ++steps;
      stage = 1;
    } else {
      ++stage;
    }
  }
  if (b == 0 && tid == 0) {
    dsc->time = time;
    dsc->dt = dt;
    dsc->steps = steps;
    dsc->alphamax = am;
    dsc->solve_pause = pause;
    if (err) atomicOr(&dsc->error, err);
  }
}

}  // namespace

bool solve1d_shape(const Params& p, Solve1dShape* sh) {
  if (p.g.ndim != 1 || p.quad || p.precision != SWFD_PRECISION_FP64) return false;
  int dev = 0, sms = 0, coop = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (sms <= 0 || !coop) return false;
  const int LI = p.g.LI;
  int cells = std::max(SWFD_SOLVE1D_MIN_CELLS, (LI + sms - 1) / sms);
  if (const char* env = getenv("SWFD_SOLVE1D_CELLS")) cells = std::max(cells, atoi(env));
  if (cells > SWFD_SOLVE1D_MAX_CELLS) return false;
  // eight lanes per flux cell (cells + 2 of them)
  const int block = (8 * (cells + 2) + 31) / 32 * 32;
  sh->cells = cells;
  sh->block = block;
  sh->grid = (LI + cells - 1) / cells;
  sh->smem = (size_t)(6 * (cells + 6) + (6 + S1_EIG) * (cells + 2) + 3 * cells) * sizeof(double);
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve1d, block, sh->smem) !=
          cudaSuccess ||
      per * sms < sh->grid)
    return false;
  return true;
}

cudaError_t launch_solve1d(const Params& p, const Solve1dShape& sh, const Solve1dArgs& a,
                           DevScalars* dsc, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(a.bar, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  Params pp = p;
  Solve1dArgs aa = a;
  DevScalars* d = dsc;
  double t_loop = p.t_loop;
  void* args[] = {&pp, &aa, &d, &t_loop};
  return cudaLaunchCooperativeKernel((const void*)k_solve1d, dim3(sh.grid), dim3(sh.block), args,
                                     sh.smem, s);
}

}  // namespace swfd
