// swfd_solve1d.cu -- the 1D point-energy solve (ex2_sedov_1d/main.f90: the
// time loop :38-53 over the SSP-RK3 step rk3 :287-328) as one persistent kernel.
//
// An 800-cell stage is a few microseconds of dependent FP64 chains; as four
// graph kernels per stage (findalpha, splitting, fluxes, RK stage) its time
// is the kernels' launch and drain latencies.  Here a cooperative grid of
// one block per SM runs the whole time loop.  Each block owns a contiguous
// range of cells.  Per stage it splits its range plus a three-cell halo in
// shared memory (dividing the stored fflux of each cell by the new
// alphamax), forms the interface fluxes of its range plus one on each side
// (reading the stored eigenvectors), and the RK stage of its own cells;
// then, on four warps side by side, checkpositivity and the next findalpha
// term (folded into the grid reduction, then the grid barrier) and the
// eigenvectors and fflux of its cells' new state (stored for the next stage,
// published to the neighbours by the block's ready flag).  A stage whose
// state fails checkpositivity ends the launch: the host runs sweep_lim on
// it and launches again at the next stage.
//
// Every value is computed by the separate kernels' code (swfd_1d.cuh).
#include "swfd_1d.cuh"
#include "swfd_gridsync.cuh"

namespace swfd {
namespace {

// a grid barrier gives up after 2 s of waiting (the slowest legitimate wait
// is one stage of the other blocks, microseconds)
constexpr unsigned long long S1_WAIT_NS = 2000000000ull;

// an interface's eigenvectors (S1_EIG values, `stride` apart)
constexpr int S1_EIG = 15;
__device__ __forceinline__ void s1_eig_store(const Eigen1D<double>& E, double* s, int stride,
                                             int j) {
  const double v[6] = {E.vxm, E.qm, E.r10, E.r12, E.r20, E.r22};
#pragma unroll
  for (int k = 0; k < 6; ++k) s[k * stride + j] = v[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) s[(6 + k) * stride + j] = E.L[k / 3][k % 3];
}
__device__ __forceinline__ void s1_eig_load(Eigen1D<double>& E, const double* s, int stride,
                                            int j) {
  E.vxm = s[j], E.qm = s[stride + j], E.r10 = s[2 * stride + j], E.r12 = s[3 * stride + j];
  E.r20 = s[4 * stride + j], E.r22 = s[5 * stride + j];
#pragma unroll
  for (int k = 0; k < 9; ++k) E.L[k / 3][k % 3] = s[(6 + k) * stride + j];
}

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

// Grid barrier k with the grid's maximum alpha and positivity flag: every
// block folds its maximum (alpha >= 0, so the bit patterns order as the
// values do) and flag into slot k % 3 before it arrives; after the barrier
// every block reads the slot.  Block 0 clears slot (k + 2) % 3 -- read by
// every block before it arrived at barrier k, next filled after barrier
// k + 1.  Returns false when the barrier's wait ran out.
__device__ __forceinline__ bool s1_sync_reduce(const Solve1dArgs& a, unsigned k, int* err,
                                               double v, int f, double& am, int& bad) {
  __shared__ double sa;
  __shared__ int sb;
  Solve1dSlot* sl = a.slots + k % 3;
  if (threadIdx.x == 0) {
    atomicMax(&sl->abits, (unsigned long long)__double_as_longlong(v));
    if (f) atomicOr(&sl->bad, 1);
  }
  if (!grid_barrier(a.bar, k, err, S1_WAIT_NS)) return false;
  if (threadIdx.x == 0) {
    sa = __longlong_as_double((long long)*(volatile unsigned long long*)&sl->abits);
    sb = *(volatile int*)&sl->bad;
    if (blockIdx.x == 0) {
      Solve1dSlot* old = a.slots + (k + 2) % 3;
      old->abits = 0;
      old->bad = 0;
    }
  }
  __syncthreads();
  am = sa;
  bad = sb;
  __syncthreads();  // sa, sb are rewritten by the next call
  return true;
}

// The same on the block's first two warps only (named barrier 1): their
// maximum v and flag f go to slot k % 3, the grid barrier passes, and
// *am, *bad (shared) receive the grid's values.  Returns false when the
// barrier's wait ran out.
__device__ __forceinline__ bool s1_sync_reduce_2w(const Solve1dArgs& a, unsigned k, int* err,
                                                  double v, int f, double* am, int* bad) {
  __shared__ double wv[2];
  __shared__ int wf[2];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  f = __any_sync(0xffffffffu, f);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) wv[w] = v, wf[w] = f;
  bar_named(1, 64);
  Solve1dSlot* sl = a.slots + k % 3;
  if (threadIdx.x == 0) {
    atomicMax(&sl->abits, (unsigned long long)__double_as_longlong(fmax(wv[0], wv[1])));
    if (wf[0] | wf[1]) atomicOr(&sl->bad, 1);
  }
  if (!grid_barrier_part(a.bar, k, err, S1_WAIT_NS, 1, 64)) return false;
  if (threadIdx.x == 0) {
    *am = __longlong_as_double((long long)*(volatile unsigned long long*)&sl->abits);
    *bad = *(volatile int*)&sl->bad;
    if (blockIdx.x == 0) {
      Solve1dSlot* old = a.slots + (k + 2) % 3;
      old->abits = 0;
      old->bad = 0;
    }
  }
  return true;
}

// the block's neighbours have published the terms of epoch e (thread 0)
__device__ __forceinline__ bool s1_wait_neighbours(const Solve1dArgs& a, unsigned e, int* err) {
  const int b = blockIdx.x;
  if (b > 0 && !wait_flag(a.ready + b - 1, e, err, S1_WAIT_NS)) return false;
  if (b + 1 < (int)gridDim.x && !wait_flag(a.ready + b + 1, e, err, S1_WAIT_NS)) return false;
  return true;
}

// a cell's precomputed terms: fflux (3 doubles) and the eigenvectors
constexpr int S1_PRE = 3 + S1_EIG;
static_assert(S1_PRE == SWFD_SOLVE1D_PRE, "the scratch's per-cell terms");

// The state buffers: st[0] = X (the step's start, u0, written back by stage
// 3), st[1] = Y, st[2] = Z; stage k reads st[k-1] and writes st[k % 3]
// (the rotation of the separate kernels' step).  The buffers change during
// the launch, so they are read with coherent loads.
//
// A GB300 SM sub-partition retires one warp-wide FP64 instruction per ~64
// cycles whatever the warp's active lanes, so a stage's time is the FP64
// instruction count of the warps on its critical path.  Each stage ends with
// the block's four warps side by side: checkpositivity, the next findalpha
// term, the eigenvectors and fflux of its cells' new state (stored for the
// next stage's split and fluxes, its own and its neighbours'); after the
// barrier only the division by the new alphamax is left of the splitting.
__global__ void __launch_bounds__(SWFD_SOLVE1D_MAX_BLOCK)
    k_solve1d(Params p, Solve1dArgs a, DevScalars* dsc, double t_loop) {
  extern __shared__ double sm[];
  const Geom& g = p.g;
  const int n = g.nx, LI = g.LI;
  const int64_t P = g.plane;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // owned cells [a0, a1) (offsets: cell i at i + 2), interface-flux cells
  // [f0, f1] within 2..n+3 (the reference's m = 0..n+1), split cells
  // [f0 - 2, f1 + 2]
  const int a0 = b * a.cells, a1 = min(LI, a0 + a.cells), nown = a1 - a0;
  const int f0 = max(a0 - 1, 2), f1 = min(a1, n + 3);
  const int nf = f1 - f0 + 1, s0 = f0 - 2, ns = nf + 4;
  const int SW = a.cells + 6, FW = a.cells + 2;
  double* ssp = sm;            // split: fp 0..2, fn 3..5, 6 x SW
  double* sfl = ssp + 6 * SW;  // interface fluxes: hp 0..2, hn 3..5, 6 x FW
  double* sev = sfl + 6 * FW;  // eigenvectors of the flux cells, S1_EIG x FW
  double* snew = sev + S1_EIG * FW;  // the stage's new state of the owned cells, 3 x cells
  // the split runs on threads [0, ns), the eigenvector copies on the warps
  // after them, threads [ev0, ev0 + nf)
  const int ev0 = (ns + 31) & ~31;
  const double* u0 = a.st[0];
  const bool sweeps = a.sweeps != 0;

  double time = dsc->time, dt = dsc->dt, am = 0.0, am_next = 0.0;
  long long steps = dsc->steps;
  const long long lim = dsc->steps_limit;
  int err = 0, pause = 0, pb = 0;
  unsigned nbar = 0, epoch = 0;  // grid barriers passed; terms published
  bool have_pre = false;
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
    if (!have_pre) {
      // findalpha (:273-285), eigenvectors and fflux of the owned cells of
      // the stage's input, on three warps
      double v = 0.0;
      for (int t = lane; t < nown; t += 32) {
        const int q = a0 + t;
        const double u1 = in[q], u2 = in[P + q], u3 = in[2 * P + q];
        if (warp == 0) {
          v = fmax(v, fmax(0.0, alpha1d(p, u1, u2, u3)));
        } else if (warp == 1 || warp == 2) {
          double* pre = a.pre + ((int64_t)pb * LI + q) * S1_PRE;
          if (warp == 1) {
            Eigen1D<double> E;
            eigen1d<double>(p.gamma1, u1, u2, u3, E);
            s1_eig_store(E, pre + 3, 1, 0);
          } else {
            double f[3];
            fflux1d(p, u1, u2, u3, f);
            for (int c = 0; c < 3; ++c) pre[c] = f[c];
          }
        }
      }
      int unused = 0;
      s1_block_reduce(v, unused);  // (a block barrier: the terms are stored)
      ++epoch;
      if (tid == 0) {
        __threadfence();
        st_release_u32(a.ready + b, epoch);
      }
      if (!s1_sync_reduce(a, ++nbar, &dsc->error, v, 0, am, unused)) return;
    } else {
      am = am_next;
    }
    {  // the neighbours' terms of this stage (their ready flags)
      __shared__ int nok;
      if (tid == 0) nok = s1_wait_neighbours(a, epoch, &dsc->error) ? 1 : 0;
      __syncthreads();
      if (!nok) return;
    }
    if (!isfinite(am) || !(am > 0.0)) err |= ERR_BIT_ALPHA;
    if (stage == 1) {  // dt = dx*cfl/alphamax (:293)
      dt = p.dt_num_x / am;
      if (!isfinite(dt)) err |= ERR_BIT_DT;
    }
    const double* pre = a.pre + (int64_t)pb * LI * S1_PRE;
    if (tid < ns) {  // the split (:82-85) of cells s0 .. s0 + ns - 1 from their fflux
      const int q = s0 + tid;
      const double u[3] = {in[q], in[P + q], in[2 * P + q]};
      const double* pq = pre + (int64_t)q * S1_PRE;
      const double f[3] = {pq[0], pq[1], pq[2]};
      double sp[3], sn[3];
      split1d_f<double>(u, f, am, sp, sn);
      for (int c = 0; c < 3; ++c) ssp[c * SW + tid] = sp[c], ssp[(3 + c) * SW + tid] = sn[c];
    } else if (tid >= ev0 && tid < ev0 + nf) {  // the flux cells' eigenvectors (:103-133)
      const int j = tid - ev0;
      const double* pq = pre + (int64_t)(f0 + j) * S1_PRE + 3;
      for (int k = 0; k < S1_EIG; ++k) sev[k * FW + j] = pq[k];
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
    {  // scheme (:252-271) and the RK stage of the owned cells, four lanes per
       // cell (lane c < 3: component c)
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
    // the new state of the owned cells: warps 0 and 1 checkpositivity
    // (:376-392) and the next findalpha term, then the grid barrier that
    // reduces them; warps 2 and 3 meanwhile the eigenvectors and fflux the
    // next stage splits and reconstructs from, published to the neighbours
    // by the block's ready flag (epoch)
    __shared__ double s_am;
    __shared__ int s_tag, s_ok;
    ++epoch;
    if (warp < 2) {
      double av = 0.0;
      int bad = 0;
      for (int t = lane; t < nown; t += 32) {
        const double n0 = snew[t], n1 = snew[a.cells + t], n2 = snew[2 * a.cells + t];
        const int q = a0 + t;
        if (warp == 0) {
          if (q - 2 >= 1 && q - 2 <= n) bad |= pos1d_bad<double>(p, n0, n1, n2);
        } else {
          av = fmax(av, fmax(0.0, alpha1d(p, n0, n1, n2)));
        }
      }
      const bool ok = s1_sync_reduce_2w(a, ++nbar, &dsc->error, av, bad, &s_am, &s_tag);
      if (tid == 0) s_ok = ok ? 1 : 0;
    } else {
      ++nbar;  // the block's grid-barrier count, as warps 0 and 1 keep it
      if (warp < 4) {
        for (int t = lane; t < nown; t += 32) {
          const double n0 = snew[t], n1 = snew[a.cells + t], n2 = snew[2 * a.cells + t];
          double* pq = a.pre + ((int64_t)(pb ^ 1) * LI + a0 + t) * S1_PRE;
          if (warp == 2) {
            Eigen1D<double> E;
            eigen1d<double>(p.gamma1, n0, n1, n2, E);
            s1_eig_store(E, pq + 3, 1, 0);
          } else {
            double f[3];
            fflux1d(p, n0, n1, n2, f);
            for (int c = 0; c < 3; ++c) pq[c] = f[c];
          }
        }
        bar_named(2, 64);
        if (tid == 64) {
          __threadfence();
          st_release_u32(a.ready + b, epoch);
        }
      }
    }
    if (tid == 0 && b == 0) dsc->rk_runs[stage]++;
    __syncthreads();
    if (!s_ok) return;
    am_next = s_am;
    const int postag = s_tag;
    __syncthreads();  // s_am, s_tag, s_ok are rewritten by the next stage
    pb ^= 1;
    have_pre = true;
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
  // eight lanes per flux cell (cells + 2 of them), and at least the four
  // warps of a stage's last phase
  const int block = std::max(128, (8 * (cells + 2) + 31) / 32 * 32);
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
  cudaError_t e = cudaMemsetAsync(a.slots, 0, 3 * sizeof(Solve1dSlot), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.bar, 0, sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.ready, 0, sh.grid * sizeof(unsigned), s);
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
