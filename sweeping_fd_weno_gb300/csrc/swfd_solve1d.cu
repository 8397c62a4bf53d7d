// swfd_solve1d.cu -- the 1D point-energy solve (ex2_sedov_1d/main.f90: the
// time loop :38-53 over the SSP-RK3 step rk3 :287-328) as one persistent kernel.
//
// An 800-cell stage is a few microseconds of dependent FP64 chains; as four
// graph kernels per stage (findalpha, splitting, fluxes, RK stage) its time
// is the kernels' launch and drain latencies.  Here a cooperative grid of
// one block per SM runs the whole time loop.  Each block owns a contiguous
// range of cells and keeps everything a stage reads in shared memory: the
// state and fflux of its range plus a three-cell halo, and the eigenvectors
// of its flux cells.  Per stage it splits (dividing the fflux by the new
// alphamax), forms the interface fluxes of its range plus one on each side,
// and the RK stage of its own cells; then, on four warps side by side,
// checkpositivity and the next findalpha term (posted to the grid reduction)
// beside the eigenvectors and fflux of its cells' new state (kept for the
// block itself and stored in global memory for its neighbours, who are told
// by the block's ready flag); those two warps then wait for the neighbours'
// flags and copy the next stage's halo into shared memory.  A stage whose
// state fails checkpositivity ends the launch: the host runs sweep_lim on it
// and launches again at the next stage.
//
// Every value is computed by the separate kernels' code (swfd_1d.cuh).
#include "swfd_1d.cuh"
#include "swfd_gridsync.cuh"

namespace swfd {
namespace {

// a wait gives up after 2 s (the slowest legitimate wait is one stage of
// the other blocks, microseconds)
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

// a cell's precomputed terms: fflux (3 doubles) and the eigenvectors
constexpr int S1_PRE = 3 + S1_EIG;
static_assert(S1_PRE == SWFD_SOLVE1D_PRE, "the scratch's per-cell terms");

// The state buffers: st[0] = X (the step's start, u0, written back by stage
// 3), st[1] = Y, st[2] = Z; stage k reads st[k-1] and writes st[k % 3]
// (the rotation of the separate kernels' step).
//
// A GB300 SM sub-partition retires one warp-wide FP64 instruction per ~64
// cycles whatever the warp's active lanes, so a stage's time is the FP64
// instruction count of the warps on its critical path plus the latency of
// its memory round trips.  Between two grid reductions a block reads global
// memory only for the halo (after the neighbours' flags, beside the grid
// reduction) and for u0 after a resume; the interface fluxes run on all
// four sub-partitions (two lanes per reconstruction).
__global__ void __launch_bounds__(SWFD_SOLVE1D_MAX_BLOCK)
    k_solve1d(Params p, Solve1dArgs a, DevScalars* dsc, double t_loop) {
  extern __shared__ double sm[];
  const Geom& g = p.g;
  const int n = g.nx, LI = g.LI;
  const int64_t P = g.plane;
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int G = gridDim.x;
  // owned cells [a0, a1), flux cells [f0, f1], split cells [s0, f1 + 2],
  // of which [s0, a0) and [a1, f1 + 2] are the halo (solve1d_layout)
  const Solve1dLayout L = solve1d_layout(b, a.cells, LI, n);
  const int a0 = L.a0, a1 = L.a1, nown = L.nown, f0 = L.f0, f1 = L.f1;
  const int nf = L.nf, s0 = L.s0, ns = L.ns, nhl = L.nhl, nhr = L.nhr;
  const int SW = a.cells + 6, FW = a.cells + 2;
  double* sst = sm;                 // state of the split cells, 3 x SW
  double* sff = sst + 3 * SW;       // their fflux, 3 x SW (right after sst)
  double* ssp = sff + 3 * SW;       // split: fp 0..2, fn 3..5, 6 x SW
  double* sfl = ssp + 6 * SW;       // interface fluxes: hp 0..2, hn 3..5, 6 x FW
  double* sev = sfl + 6 * FW;       // eigenvectors of the flux cells, S1_EIG x FW
  double* su0 = sev + S1_EIG * FW;  // u0 of the owned cells, 3 x cells
  __shared__ double s_am;
  __shared__ int s_tag, s_ok, s_nok[2];
  const bool sweeps = a.sweeps != 0;

  double time = dsc->time, dt = dsc->dt, am = 0.0;
  long long steps = dsc->steps;
  const long long lim = dsc->steps_limit;
  int err = 0, pause = 0, pw = 0;
  unsigned nred = 0, epoch = 0;  // grid reductions passed; terms published
  bool after = false;            // the terms follow a stage (else the launch's start)
  bool u0_ok = false;            // su0 holds u0 (a stage 1 ran in this launch)
  int stage = a.resume;
  if (stage == 4) {  // the step whose stage-3 sweep the host ran: time = time + dt (:44)
    time = time + dt;
    ++steps;
    stage = 1;
  }
  // the launch starts from the state stage `stage` reads: its owned cells
  const double* src = a.st[stage - 1];
  for (int w = tid; w < 3 * nown; w += blockDim.x) {
    const int c = w / nown, t = w - c * nown;
    sst[c * SW + a0 + t - s0] = src[c * P + a0 + t];
  }
  __syncthreads();
  for (;;) {
    // ---- the terms of the state in sst (owned cells; src in global memory)
    // for the next stage: warps 0 and 1 checkpositivity (:376-392, after a
    // stage) and findalpha (:273-285), then the grid reduction; warps 2 and
    // 3 the eigenvectors (:103-133) and fflux (:57-73), kept and published
    // to the neighbours (ready flag), then the neighbours' halo
    ++epoch;
    ++nred;
    if (warp < 2) {
      unsigned long long ab = 0;
      int bad = 0;
      for (int t = lane; t < nown; t += 32) {
        const int q = a0 + t, tt = q - s0;
        const double n0 = sst[tt], n1 = sst[SW + tt], n2 = sst[2 * SW + tt];
        if (warp == 0) {
          if (after && q - 2 >= 1 && q - 2 <= n) bad |= pos1d_bad<double>(p, n0, n1, n2);
        } else {
          const double al = fmax(0.0, alpha1d(p, n0, n1, n2));
          ab = umax64(ab, (unsigned long long)__double_as_longlong(al) & ~GRID_WORD_BAD);
        }
      }
      // the release half of thread 0's post (see grid_reduce_2w), beside warp 1's findalpha
      if (tid == 0) fence_acq_rel_gpu();
      const bool ok =
          grid_reduce_2w(a.red, nred, &dsc->error, S1_WAIT_NS, ab, bad, &s_am, &s_tag);
      if (tid == 0) s_ok = ok ? 1 : 0;
    } else if (warp < 4) {
      double* prew = a.pre + (int64_t)pw * LI * S1_PRE;
      for (int t = lane; t < nown; t += 32) {
        const int q = a0 + t, tt = q - s0;
        const double n0 = sst[tt], n1 = sst[SW + tt], n2 = sst[2 * SW + tt];
        double* pq = prew + (int64_t)q * S1_PRE;
        if (warp == 2) {
          Eigen1D<double> E;
          eigen1d<double>(p.gamma1, n0, n1, n2, E);
          s1_eig_store(E, pq + 3, 1, 0);
          if (q >= f0 && q <= f1) s1_eig_store(E, sev, FW, q - f0);
        } else {
          double f[3];
          fflux1d(p, n0, n1, n2, f);
#pragma unroll
          for (int c = 0; c < 3; ++c) pq[c] = f[c], sff[c * SW + tt] = f[c];
        }
      }
      bar_named(2, 64);
      // the release store orders the block's stores of the state (before
      // the block barrier after the RK stage) and of the terms (before the
      // named barrier) before the flag
      if (tid == 64) st_release_u32(a.ready + b, epoch);
      if (tid == 64 || tid == 96) {  // the left and the right neighbour, side by side
        const int nb = tid == 64 ? b - 1 : b + 1;
        int okn = 1;
        if (nb >= 0 && nb < G) okn = wait_flag(a.ready + nb, epoch, &dsc->error, S1_WAIT_NS);
        s_nok[tid == 96] = okn;
      }
      bar_named(2, 64);
      if (s_nok[0] && s_nok[1]) {
        // the halo, all loads first: thread 64 + t2 takes value t2 of the
        // halo cells' state (from src) and fflux (six per cell), and value
        // 63 - t2 of the eigenvectors of the flux cells next to the range
        // (f0 below a0: 0..14, f1 at a1: 15..29)
        const int t2 = tid - 64;
        const bool hasA = t2 < 6 * (nhl + nhr);
        const int eB = 63 - t2;
        const bool right = eB >= S1_EIG;
        const int qB = right ? f1 : f0, kB = eB - (right ? S1_EIG : 0);
        const bool hasB = eB < 2 * S1_EIG && (right ? f1 >= a1 : f0 < a0);
        double vA = 0.0, vB = 0.0;
        int dA = 0;
        if (hasA) {
          const int ci = t2 / 6, comp = t2 - 6 * ci;
          const int q = ci < nhl ? s0 + ci : a1 + (ci - nhl);
          dA = comp * SW + q - s0;  // comp 3..5 land in sff
          vA = comp < 3 ? __ldcg(src + comp * P + q)
                        : __ldcg(prew + (int64_t)q * S1_PRE + (comp - 3));
        }
        if (hasB) vB = __ldcg(prew + (int64_t)qB * S1_PRE + 3 + kB);
        if (hasA) sst[dA] = vA;
        if (hasB) sev[kB * FW + qB - f0] = vB;
      }
    }
    __syncthreads();
    if (!s_ok || !s_nok[0] || !s_nok[1]) return;
    const double am_next = s_am;
    const int postag = s_tag;
    pw ^= 1;
    if (after) {
      if (tid == 0 && b == 0) dsc->rk_runs[stage]++;
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
    // ---- stage `stage`: DO WHILE (time <= time_terminal - 1d-10), within
    // the launch's step bound
    if (stage == 1 && !(time <= t_loop && steps < lim && err == 0)) break;
    am = am_next;
    double* out = a.st[stage % 3];
    if (!isfinite(am) || !(am > 0.0)) err |= ERR_BIT_ALPHA;
    if (stage == 1) {  // dt = dx*cfl/alphamax (:293)
      dt = p.dt_num_x / am;
      if (!isfinite(dt)) err |= ERR_BIT_DT;
    }
    {  // the split (:82-85) of cells s0 .. s0 + ns - 1 from their fflux, one
       // component per warp (ns <= 32) or group of warps
      const int nsr = (ns + 31) & ~31;
      for (int w = tid; w < 3 * nsr; w += blockDim.x) {
        const int c = w / nsr, t = w - c * nsr;
        if (t < ns) {
          double sp, sn;
          split1d_one(sst[c * SW + t], sff[c * SW + t], am, sp, sn);
          ssp[c * SW + t] = sp;
          ssp[(3 + c) * SW + t] = sn;
        }
      }
    }
    __syncthreads();
    // interface fluxes (:88-157), sixteen lanes per flux cell f0 + j
    for (int jb = 0; jb < nf; jb += (int)(blockDim.x >> 4)) {
      const int j = jb + (tid >> 4), sub = tid & 15;
      const int jc = j < nf ? j : max(nf - 1, 0);  // lanes past the range repeat the last cell
      Eigen1D<double> E;
      s1_eig_load(E, sev, FW, jc);
      const double v = recon1d_pair(
          p, E, sub, [&](int side, int c, int jj) { return ssp[(3 * side + c) * SW + jc + jj]; });
      const double r = back1d<double, 16>(E, v, sub);
      if (!p.limiter) {
        if (j < nf && sub < 6) sfl[sub * FW + j] = r;
      } else {  // use_limiter 1 (:159-245): lanes 0 and 3 limit their side
        double w[3];
        int nd = 0, np = 0;
        const bool lim1 = limit1d_group<double, 16>(
            p, r, sub, [&](int side, int c) { return ssp[(3 * side + c) * SW + jc + 2]; }, w, nd,
            np);
        if (j < nf && lim1) {
#pragma unroll
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
       // cell (lane c < 3: component c); the new state replaces the stage's
       // input in sst (each value read and written by one thread)
      const int cell = tid >> 2, c = tid & 3, q = a0 + cell;
      const int i = q - 2;
      if (cell < nown && c < 3) {
        const int tt = q - s0;
        const double uin = sst[c * SW + tt];
        double r = 0.0;
        if (i >= 1 && i <= n) {
          const int k = q - f0;
          r = rhs1d_value<double>(p, am, sfl[c * FW + k - 1], sfl[(3 + c) * FW + k],
                                  sfl[c * FW + k], sfl[(3 + c) * FW + k + 1]);
        }
        const double u0v =
            stage == 1 ? uin : u0_ok ? su0[c * a.cells + cell] : a.st[0][c * P + q];
        const double v = rk1d_value<double>(p, stage, dt, r, uin, &u0v);
        out[c * P + q] = v;
        sst[c * SW + tt] = v;
        if (stage == 1) su0[c * a.cells + cell] = uin;
      }
    }
    if (stage == 1) u0_ok = true;
    __syncthreads();
    src = out;
    after = true;
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
  // sixteen lanes per flux cell (cells + 2 of them; more take turns), four
  // per owned cell in the RK stage, and at least the four warps of the
  // terms of a stage
  const int block =
      std::min(SWFD_SOLVE1D_MAX_BLOCK, std::max(128, (16 * (cells + 2) + 31) / 32 * 32));
  sh->cells = cells;
  sh->block = block;
  sh->grid = (LI + cells - 1) / cells;
  if (sh->grid > 64 * SWFD_SOLVE1D_POLL || 4 * cells > block) return false;
  sh->smem = (size_t)(12 * (cells + 6) + (6 + S1_EIG) * (cells + 2) + 3 * cells) * sizeof(double);
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_solve1d, block, sh->smem) !=
          cudaSuccess ||
      per * sms < sh->grid)
    return false;
  return true;
}

cudaError_t launch_solve1d(const Params& p, const Solve1dShape& sh, const Solve1dArgs& a,
                           DevScalars* dsc, cudaStream_t s) {
  // the reduction words empty (all ones), the ready flags zero
  cudaError_t e = cudaMemsetAsync(
      a.red, 0xff, 3 * (size_t)sh.grid * SWFD_SOLVE1D_WSTRIDE * sizeof(unsigned long long), s);
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
