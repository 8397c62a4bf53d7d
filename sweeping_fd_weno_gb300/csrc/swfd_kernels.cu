// swfd_kernels.cu -- boundary conditions, CFL reduction, LF splitting, the
// characteristic WENO5 interface fluxes and the fused RHS + SSP-RK3 update.
#include "swfd_1d.cuh"

namespace swfd {

#define SWFD_BLOCK 256

__device__ __forceinline__ double ld(const double* p) { return __ldg(p); }
// NC: the read-only (non-coherent) path; false for values this kernel may
// have written itself
template <bool NC>
__device__ __forceinline__ double ldc(const double* p) {
  if constexpr (NC) return __ldg(p);
  else return *p;
}

// ---------------------------------------------------------------------------
// bc: every ghost cell gets its final value directly, resolved through the
// order in which the reference applies its loops (the order defines the
// corner ghosts).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void bc2d_cell(const Params& p, double* __restrict__ u, int64_t t) {
  const Geom& g = p.g;
  const int nx = g.nx, ny = g.ny;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  if (t >= ncell) return;
  int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  bool gi = (i < 1 || i > nx), gj = (j < 1 || j > ny);
  if (p.problem == SWFD_PROBLEM_SHOCK_DIFFRACTION) {
    // ex6_shock_diffraction/main.f90:895-940 in its order: fixed bottom rows,
    // fixed right columns, top rows copied from row ny, inflow left columns,
    // then the quiescent column i = 1 (the DO variable after `do i = -2, 0`)
    // below row 6*total.  The rank exchanges before them only fill ghosts
    // that these overwrite, or interior cells of the single grid.
    const double gm = p.gamma, g1 = p.gamma1;
    double w[4] = {gm, 0., 0., 1. / g1};
    if (i == 1 && j < 6 * p.total) {
      w[0] = 1.;
    } else if (i <= 0) {
      for (int c = 0; c < 4; ++c) w[c] = p.inflow[c];
    } else if (i > nx || j <= 0) {
      // fixed state
    } else if (j > ny) {
      for (int c = 0; c < 4; ++c) w[c] = u[c * g.plane + g.at(i, ny)];
    } else {
      return;
    }
    const int64_t o = g.at(i, j);
    for (int c = 0; c < 4; ++c) u[c * g.plane + o] = w[c];
    return;
  }
  if (!gi && !gj) return;
  double v[4];
  int si = i, sj = j;
  double sgn[4] = {1., 1., 1., 1.};
  bool fixed = false;
  if (p.problem == SWFD_PROBLEM_VORTEX_2D) {
    // ex3_vortex_accuracy_2d/main.f90:653-669: x wrap for all rows, then y
    // wrap for all columns -> fully periodic
    si = i < 1 ? i + nx : (i > nx ? i - nx : i);
    sj = j < 1 ? j + ny : (j > ny ? j - ny : j);
  } else {
    // ex4_sedov_2d/main.f90:922-994, ex5_mach2000_jet/main.f90:702-738:
    // left (reflect / inflow) for all rows, bottom reflect for all columns,
    // right outflow for all rows, top outflow for all columns.
    const bool jet = (p.problem == SWFD_PROBLEM_JET_2D);
    int ii = i, jj = j;
    if (jj > ny) jj = ny;             // top outflow copies row ny
    if (ii > nx) ii = nx;             // right outflow copies column nx
    if (jj < 1) {
      if (p.jet_full) {               // full-domain jet: bottom outflow copies row 1
        jj = 1;
      } else {                        // bottom reflect of row 1-j
        jj = 1 - jj;
        sgn[2] = -1.;
      }
    }
    if (ii < 1) {
      if (jet) {
        // inflow state of row jj, then (if jj came from the bottom) mirrored
        const double* s = (jj >= p.jet_jmin && jj <= p.jet_jmax) ? p.jet_in : p.jet_amb;
        for (int c = 0; c < 4; ++c) v[c] = s[c];
        fixed = true;
      } else {
        ii = 1 - ii;                  // left reflect
        sgn[1] = -1.;
      }
    }
    si = ii;
    sj = jj;
  }
  if (!fixed)
    for (int c = 0; c < 4; ++c) v[c] = u[c * g.plane + g.at(si, sj)];
  const int64_t o = g.at(i, j);
  for (int c = 0; c < 4; ++c) u[c * g.plane + o] = (sgn[c] < 0.) ? -v[c] : v[c];
}

__global__ void k_bc2d(Params p, double* __restrict__ u) {
  bc2d_cell(p, u, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

cudaError_t launch_bc(const Params& p, double* u, cudaStream_t s) {
  if (p.g.ndim == 1) return cudaSuccess;  // ex2_sedov_1d/main.f90:394-403 is empty
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  k_bc2d<<<(unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(p, u);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// findalpha: max over all cells including ghosts
// ---------------------------------------------------------------------------
__device__ __forceinline__ double block_max(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;
}

// F32: the FP32-bulk 2D form only (the fused FP32 kernels), so that the
// other forms' code -- and its registers -- stay out of those kernels
template <bool NC = true, bool F32 = false>
__device__ __forceinline__ double alpha_cell(const Params& p, const double* __restrict__ u,
                                             int64_t t) {
  const Geom& g = p.g;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  double a = 0.0;
  if (t < ncell) {
    int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
    int64_t o = g.at(i, j);
    const double g1 = p.gamma1, gamma = p.gamma;
    if (!F32 && g.ndim == 1) {
      // ex2_sedov_1d/main.f90:278-283
      a = alpha1d(p, ldc<NC>(u + o), ldc<NC>(u + g.plane + o), ldc<NC>(u + 2 * g.plane + o));
    } else if (F32 || p.precision == SWFD_PRECISION_FP32_BULK) {
      // FP32-bulk: the pressure recovered in FP64 (one reciprocal per cell);
      // the CFL quantities (velocities, sound speed, their max) in FP32
      double u1 = ldc<NC>(u + o), u2 = ldc<NC>(u + g.plane + o), u3 = ldc<NC>(u + 2 * g.plane + o),
             u4 = ldc<NC>(u + 3 * g.plane + o);
      const double ri = rcp_bulk(u1);
      double pres;
      if (!p.alpha_guarded) {
        pres = g1 * fma(-0.5 * ri, fma(u2, u2, u3 * u3), u4);
      } else {
        const double vx = u1 >= p.eps2 ? u2 * ri : 0., vy = u1 >= p.eps2 ? u3 * ri : 0.;
        pres = g1 * fma(-0.5 * u1, fma(vx, vx, vy * vy), u4);
      }
      const float fri = d2f(ri);
      const float sound = sqrtf(d2f(gamma) * d2f(pres) * fri);
      a = f2d(fmaxf(fabsf(d2f(u2) * fri), fabsf(d2f(u3) * fri)) + sound);
    } else if constexpr (!F32) {
      double u1 = ldc<NC>(u + o), u2 = ldc<NC>(u + g.plane + o), u3 = ldc<NC>(u + 2 * g.plane + o),
             u4 = ldc<NC>(u + 3 * g.plane + o);
      // the first quotients straight-line (they interleave), tdiv's fallback
      // for the rare operand
      int bad = 0;
      double q2 = div_nfz(u2, u1, bad), q3 = div_nfz(u3, u1, bad);
      if (!p.alpha_guarded) {
        // ex3_vortex_accuracy_2d/main.f90:556-559
        double k2 = div_nfz(u2 * u2, u1, bad), k3 = div_nfz(u3 * u3, u1, bad);
        if (bad) {
          q2 = tdiv(u2, u1), q3 = tdiv(u3, u1);
          k2 = tdiv(u2 * u2, u1), k3 = tdiv(u3 * u3, u1);
        }
        double pres = g1 * (u4 - tscale<-1>(k2) - tscale<-1>(k3));
        double sound = sqrt(tdiv(gamma * pres, u1));
        a = fmax(fabs(q2) + sound, fabs(q3) + sound);
      } else {
        // ex5_mach2000_jet/main.f90:571-584
        if (bad) q2 = tdiv(u2, u1), q3 = tdiv(u3, u1);
        double vx = 0., vy = 0.;
        if (u1 >= p.eps2) {
          vx = q2;
          vy = q3;
        }
        const double hu1 = tscale<-1>(u1);
        double pres = g1 * (u4 - hu1 * (vx * vx) - hu1 * (vy * vy));
        double sound = sqrt(tdiv(gamma * pres, u1));
        a = fmax(fabs(q2) + sound, fabs(q3) + sound);
      }
    }
    a = fmax(0.0, a);
  }
  return a;
}

// ex6 keeps every cell's alpha for the per-rank-row and per-rank-column maxima
__device__ __forceinline__ void alpha_store(const Params& p, int64_t t, double a) {
  const Geom& g = p.g;
  if (!p.alpha_plane || t >= (int64_t)g.LI * g.LJ) return;
  p.alpha_plane[g.at(((int)t % g.LI) - 2, ((int)t / g.LI) - 2)] = a;
}

__device__ __forceinline__ void alpha_final_body(DevScalars* dsc) {
  dsc->alphamax = __longlong_as_double((long long)dsc->alpha_bits);
  if (!isfinite(dsc->alphamax) || !(dsc->alphamax > 0.0)) dsc->error |= 1;
}

__device__ __forceinline__ void dt_body(const Params& p, DevScalars* dsc);

// Every block folds its maximum into alpha_bits (alpha >= 0, so the bit
// patterns order as the values do).  The last block to finish turns the
// maximum into alphamax -- and, after the stage-1 findalpha, into dt -- and
// re-arms the accumulator and the block counter for the next launch, so a
// stage needs neither a reset nor a single-thread finishing kernel.  It also
// clears postag, which the RK kernel of the same stage accumulates.
// the block's maximum a folded into alpha_bits by thread 0; the last block
// finishes the reduction (and, with_dt, the dt rule)
__device__ __forceinline__ void alpha_last_block(const Params& p, DevScalars* dsc, double a,
                                                 int with_dt) {
  atomicMax(&dsc->alpha_bits, (unsigned long long)__double_as_longlong(a));
  __threadfence();
  if (atomicAdd(&dsc->alpha_done, 1) != (int)gridDim.x - 1) return;
  __threadfence();
  const unsigned long long m = atomicExch(&dsc->alpha_bits, 0ull);
  dsc->alpha_done = 0;
  dsc->postag = 0;
  dsc->alphamax = __longlong_as_double((long long)m);
  if (!isfinite(dsc->alphamax) || !(dsc->alphamax > 0.0)) dsc->error |= 1;
  if (with_dt) dt_body(p, dsc);
}

__global__ void k_alpha(Params p, const double* __restrict__ u, DevScalars* dsc, int with_dt) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double a = alpha_cell(p, u, t);
  alpha_store(p, t, a);
  a = block_max(a);
  if (threadIdx.x != 0) return;
  alpha_last_block(p, dsc, a, with_dt);
}

// bc followed by the next stage's findalpha, in one pass over the cells: each
// thread fills its ghost cell (bc2d_cell), then takes the alpha of its cell
// from the value it just wrote (a coherent load) or, for an interior cell,
// from the state the RK stage and the sweep left; the block maxima and the
// last block's decisions are k_alpha's.  Problems with rank segments keep
// their separate findalpha (their per-cell alphas feed the per-row and
// per-column maxima).
__global__ void k_bc2d_alpha(Params p, double* __restrict__ u, DevScalars* dsc) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bc2d_cell(p, u, t);
  double a = alpha_cell<false>(p, u, t);
  a = block_max(a);
  if (threadIdx.x != 0) return;
  alpha_last_block(p, dsc, a, 0);
}

// Threads per block of the per-cell kernels: 256, or fewer (down to one warp)
// on grids too small to give every SM two blocks, so that the FP64 work of a
// small grid (2 FP64 instructions per clock per SM) spreads over the SMs.
// The per-cell results do not depend on it.
static int cell_block(int64_t cells, int bmax = SWFD_BLOCK) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  int b = bmax > 0 ? bmax : SWFD_BLOCK;
  while (b > 32 && (cells + b - 1) / b < 2 * sms) b >>= 1;
  return b;
}

cudaError_t launch_bc_alpha(const Params& p, double* u, DevScalars* dsc, cudaStream_t s) {
  const int64_t n = (int64_t)p.g.LI * p.g.LJ;
  const int b = cell_block(n);
  k_bc2d_alpha<<<(unsigned)((n + b - 1) / b), b, 0, s>>>(p, u, dsc);
  return cudaGetLastError();
}

cudaError_t launch_alpha(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s,
                         bool with_dt) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  const int b = cell_block(n);
  k_alpha<<<(unsigned)((n + b - 1) / b), b, 0, s>>>(p, u, dsc, with_dt ? 1 : 0);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// ex6: the Lax-Friedrichs alpha of each rank row (x pass) and rank column
// (y pass): the max of the per-cell alpha over the rank's local cells,
// ghosts included, starting from 0 (ex6_shock_diffraction/main.f90:218-221,
// 450-453).  One thread per (row, x segment) and per (column, y segment).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void seg_alpha_item(const Params& p, int64_t t) {
  const Geom& g = p.g;
  const int64_t nrow = (int64_t)g.LJ * p.cut_x;
  if (t < nrow) {
    const int j = ((int)t / p.cut_x) - 2, sx = ((int)t % p.cut_x);
    const int i0 = sx * p.nxl - 2, i1 = sx * p.nxl + p.nxl + 3;
    double a = 0.;
    for (int i = i0; i <= i1; ++i) a = fmax(a, p.alpha_plane[g.at(i, j)]);
    p.seg_ax[t] = a;
    return;
  }
  t -= nrow;
  if (t >= (int64_t)g.LI * p.cut_y) return;
  const int i = ((int)t / p.cut_y) - 2, sy = ((int)t % p.cut_y);
  const int j0 = sy * p.nyl - 2, j1 = sy * p.nyl + p.nyl + 3;
  double a = 0.;
  for (int j = j0; j <= j1; ++j) a = fmax(a, p.alpha_plane[g.at(i, j)]);
  p.seg_ay[t] = a;
}

__global__ void k_seg_alpha(Params p) {
  seg_alpha_item(p, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

__host__ __device__ __forceinline__ int64_t seg_alpha_items(const Params& p) {
  return (int64_t)p.g.LJ * p.cut_x + (int64_t)p.g.LI * p.cut_y;
}

// ex6 wall mirrors.  x: columns total, total-1, total-2 of rows 0..6*total
// take columns total+1..total+3 with m_x negated (:191-201); y: rows
// 6*total, -1, -2 of columns 1..total take rows 6*total+1..+3 with m_y
// negated (:416-430).  Targets and sources never overlap.
__device__ __forceinline__ void wall_x_item(const Params& p, double* __restrict__ u, int t) {
  const Geom& g = p.g;
  const int rows = min(6 * p.total, g.ny + 1) + 1;  // rows 0..min(6*total, ny+1)
  if (t >= rows * 3) return;
  const int j = t / 3, k = t % 3;
  const int64_t dst = g.at(p.total - k, j), src = g.at(p.total + 1 + k, j);
  for (int c = 0; c < 4; ++c) {
    p.wall_save[(int64_t)t * 4 + c] = u[c * g.plane + dst];
    const double v = u[c * g.plane + src];
    u[c * g.plane + dst] = (c == 1) ? -v : v;
  }
}
__device__ __forceinline__ void wall_y_item(const Params& p, double* __restrict__ u, int t) {
  const Geom& g = p.g;
  if (t >= p.total * 3) return;
  const int i = t % p.total + 1, k = t / p.total;
  const int r = 6 * p.total;
  const int64_t dst = g.at(i, r - k), src = g.at(i, r + 1 + k);
  for (int c = 0; c < 4; ++c) {
    const double v = u[c * g.plane + src];
    u[c * g.plane + dst] = (c == 2) ? -v : v;
  }
}
__global__ void k_wall_x(Params p, double* __restrict__ u) {
  wall_x_item(p, u, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_wall_y(Params p, double* __restrict__ u) {
  wall_y_item(p, u, blockIdx.x * blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------------------
// dt rule, after the stage-1 findalpha
// (ex2_sedov_1d/main.f90:293; ex3_vortex_accuracy_2d/main.f90:572;
//  ex4_sedov_2d/main.f90:696-700; ex5_mach2000_jet/main.f90:601-605)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dt_body(const Params& p, DevScalars* dsc) {
  const double am = dsc->alphamax;
  double dt;
  if (p.dt_rule == 4) {
    double dtx = p.dt_num_x / am, dty = p.dt_num_y / am;
    double dtc = fmin(dtx, dty);
    dt = fmin(dtc, p.time_terminal - dsc->time);
  } else {
    dt = p.dt_num_x / am;
  }
  dsc->dt = dt;
  if (!isfinite(dt)) dsc->error |= 2;
}

__global__ void k_time_advance(DevScalars* dsc) { dsc->time = dsc->time + dsc->dt; }

cudaError_t launch_time_advance(DevScalars* dsc, cudaStream_t s) {
  k_time_advance<<<1, 1, 0, s>>>(dsc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Lax-Friedrichs splitting + Roe preparation, one thread per cell
// (ex3_vortex_accuracy_2d/main.f90:61-131,134-147,335-348)
// split planes: [0,nc) fp, [nc,2nc) fn, [2nc,3nc) gp, [3nc,4nc) gn
// roe planes:   0 w, 1 vx, 2 vy, 3 h (x pass); 4..7 the y pass (ex4 only)
// Pressure recovery from the conserved variables is FP64 in both precisions;
// the split fluxes and Roe averages are stored and formed in T.
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T ldt(const T* p) { return __ldg(p); }

template <class T>
__device__ __forceinline__ T sqrt_abs(double v);
template <>
__device__ __forceinline__ double sqrt_abs<double>(double v) { return sqrt(fabs(v)); }
template <>
__device__ __forceinline__ float sqrt_abs<float>(double v) { return sqrtf(fabsf(d2f(v))); }

// which: 1 = x pass (fp, fn and the x Roe planes), 2 = y pass (gp, gn and,
// with the ex4 regularisers, the y Roe planes), 3 = both.  With rank
// segments (ex6) a cell near a rank boundary is split once per segment whose
// local range holds it, with that segment's alpha.
// 1/(den + 1d-15) of the y-pass preparation of ex4 and ex6
// (ex4_sedov_2d/main.f90:426); in binary128 for the QUAD build
__device__ __forceinline__ double reg_recip(const Params& p, double den) {
  if (p.quad)
    return qd::to_double(qd::div(qd::from_double(1.0), qd::add(qd::from_double(den), p.q_1em15)));
  return sd::div(1., den + 1e-15);
}

// FP32-bulk splitting of one cell (no rank segments): the pressure recovered
// in FP64 (fused multiply-adds, one reciprocal), the conserved values and the
// x and y fluxes rounded to binary32 and formed there.  The Lax-Friedrichs
// split fluxes 0.5 (a +- f/alpha) come from these nine terms through
// split_pm, whether the splitting kernel forms them or the fused stage
// kernel does in its shared-memory tile: the same operations, the same bits.
struct Terms32 {
  float fr, fm, fn, fe;  // rho, m, n, E
  float f1, fxy, f3;     // x fluxes rho u^2 + p, rho u v, (E + p) u (the first is m)
  float g2, g3;          // y fluxes rho v^2 + p, (E + p) v (the first is n, the second fxy)
};
struct Prim32 {  // FP64 velocities and pressure of the splitting (the Roe planes reuse them)
  double vx, vy, pres;
  bool guard;
};
__device__ __forceinline__ Terms32 terms32(const Params& p, double rho, double mx, double my,
                                           double e, double ri, Prim32& q) {
  double vx = mx * ri, vy = my * ri;
  q.guard = p.flux_guard_eps2 ? (rho < p.eps2) : (rho < p.lim8_lt);
  if (q.guard) vx = vy = 0.;
  q.pres = p.gamma1 * fma(-0.5 * rho, fma(vx, vx, vy * vy), e);
  q.vx = vx;
  q.vy = vy;
  Terms32 t;
  t.fr = d2f(rho), t.fm = d2f(mx), t.fn = d2f(my), t.fe = d2f(e);
  const float fvx = d2f(vx), fvy = d2f(vy), fp = d2f(q.pres);
  t.fxy = t.fr * fvx * fvy;
  t.f1 = fmaf(t.fr * fvx, fvx, fp);
  t.f3 = (t.fe + fp) * fvx;
  t.g2 = fmaf(t.fr * fvy, fvy, fp);
  t.g3 = (t.fe + fp) * fvy;
  return t;
}
// 0.5 (a + f/alpha) and 0.5 (a - f/alpha) with ram = 1/alpha, each one
// rounding of a fused multiply-add and an exact halving
__device__ __forceinline__ void split_pm(float a, float f, float ram, float& sp, float& sn) {
  sp = 0.5f * fmaf(f, ram, a);
  sn = 0.5f * fmaf(-f, ram, a);
}
// the 16 split values of a cell in the plane order of the split planes:
// fp (0..3), fn (4..7), gp (8..11), gn (12..15)
__device__ __forceinline__ void split32(const Terms32& t, float ram, float s[16]) {
  split_pm(t.fr, t.fm, ram, s[0], s[4]);
  split_pm(t.fm, t.f1, ram, s[1], s[5]);
  split_pm(t.fn, t.fxy, ram, s[2], s[6]);
  split_pm(t.fe, t.f3, ram, s[3], s[7]);
  split_pm(t.fr, t.fn, ram, s[8], s[12]);
  split_pm(t.fm, t.fxy, ram, s[9], s[13]);
  split_pm(t.fn, t.g2, ram, s[10], s[14]);
  split_pm(t.fe, t.g3, ram, s[11], s[15]);
}
// the Roe planes of the FP32-bulk preparation; the enthalpy reuses the
// recovered pressure (x pass) and, with the ex4 regularisers, the y pass has
// its own (ex4_sedov_2d/main.f90:426)
__device__ __forceinline__ void roe32_store(const Params& p, double rho, double mx, double my,
                                            double e, double ri, const Prim32& q, float fr,
                                            float* __restrict__ roe, int64_t P, int64_t o,
                                            int which) {
  const double g1 = p.gamma1;
  if (which & 1) {
    const double vex = q.guard ? mx * ri : q.vx, vey = q.guard ? my * ri : q.vy;
    const double pre = q.guard ? g1 * fma(-0.5, fma(mx, vex, my * vey), e) : q.pres;
    roe[0 * P + o] = sqrtf(fabsf(fr));
    roe[1 * P + o] = d2f(vex);
    roe[2 * P + o] = d2f(vey);
    roe[3 * P + o] = d2f((pre + e) * ri);
  }
  if (p.roe_reg_ex4 && (which & 2)) {
    const double t0 = 1. / (rho + 1e-15);
    const double vex = mx * t0, vey = my * t0;
    const double pre = g1 * fma(-0.5, fma(mx, vex, my * vey), e);
    roe[4 * P + o] = sqrtf(fabsf(fr));
    roe[5 * P + o] = d2f(vex);
    roe[6 * P + o] = d2f(vey);
    roe[7 * P + o] = d2f((pre + e) * t0);
  }
}

template <class T>
__device__ __forceinline__ void prep2d_cell(const Params& p, const double* __restrict__ u,
                                            double amd, T* __restrict__ split, T* __restrict__ roe,
                                            int64_t t, int which = 3) {
  const Geom& g = p.g;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  if (t >= ncell) return;
  int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  const int64_t o = g.at(i, j), P = g.plane;
  const double g1 = p.gamma1;
  double rho = ld(u + o), mx = ld(u + P + o), my = ld(u + 2 * P + o), e = ld(u + 3 * P + o);
  constexpr bool F32 = sizeof(T) == 4;  // FP32-bulk: FP64 with one reciprocal per cell
  const double ri = F32 ? rcp_bulk(rho) : 0.;
  if constexpr (F32) {
    if (!p.seg_alpha) {
      Prim32 q;
      const Terms32 tm = terms32(p, rho, mx, my, e, ri, q);
      const float ram = 1.f / d2f(amd);
      const int64_t S = p.sg.plane;
      float sp[16];
      split32(tm, ram, sp);
#pragma unroll
      for (int k = 0; k < 16; ++k) split[k * S + o] = sp[k];
      roe32_store(p, rho, mx, my, e, ri, q, tm.fr, roe, P, o, which);
      return;
    }
  }
  // fflux / gflux
  double vx = F32 ? mx * ri : tdiv(mx, rho), vy = F32 ? my * ri : tdiv(my, rho);
  bool guard = p.flux_guard_eps2 ? (rho < p.eps2) : (rho < p.lim8_lt);
  if (guard) {
    vx = 0.;
    vy = 0.;
  }
  const double hrho = tscale<-1>(rho);  // 0.5*rho
  double pres = g1 * (e - hrho * (vx * vx) - hrho * (vy * vy));
  double fxy = rho * vx * vy;
  double f1 = rho * (vx * vx) + pres, f3 = (e + pres) * vx;
  double g2 = rho * (vy * vy) + pres, g3 = (e + pres) * vy;
  // fp = 0.5*(u + f/alpha), fn = 0.5*(u - f/alpha); f/alpha shared by both
  const T tr = T(rho), tmx = T(mx), tmy = T(my), te = T(e);
  const int64_t S = p.sg.plane;
  if (!p.seg_alpha && F32) {
    const T ram = T(1.) / T(amd);
    T q;
    q = T(mx) * ram;  split[0 * S + o] = tscale<-1>(tr + q);   split[4 * S + o] = tscale<-1>(tr - q);
    q = T(f1) * ram;  split[1 * S + o] = tscale<-1>(tmx + q);  split[5 * S + o] = tscale<-1>(tmx - q);
    T qxy = T(fxy) * ram;
    split[2 * S + o] = tscale<-1>(tmy + qxy); split[6 * S + o] = tscale<-1>(tmy - qxy);
    q = T(f3) * ram;  split[3 * S + o] = tscale<-1>(te + q);   split[7 * S + o] = tscale<-1>(te - q);
    q = T(my) * ram;  split[8 * S + o] = tscale<-1>(tr + q);   split[12 * S + o] = tscale<-1>(tr - q);
    split[9 * S + o] = tscale<-1>(tmx + qxy); split[13 * S + o] = tscale<-1>(tmx - qxy);
    q = T(g2) * ram;  split[10 * S + o] = tscale<-1>(tmy + q); split[14 * S + o] = tscale<-1>(tmy - q);
    q = T(g3) * ram;  split[11 * S + o] = tscale<-1>(te + q);  split[15 * S + o] = tscale<-1>(te - q);
  } else if (!p.seg_alpha) {
    const T am = T(amd);
    T q;
    q = tdiv(T(mx), am);  split[0 * S + o] = tscale<-1>(tr + q);   split[4 * S + o] = tscale<-1>(tr - q);
    q = tdiv(T(f1), am);  split[1 * S + o] = tscale<-1>(tmx + q);  split[5 * S + o] = tscale<-1>(tmx - q);
    T qxy = tdiv(T(fxy), am);
    split[2 * S + o] = tscale<-1>(tmy + qxy); split[6 * S + o] = tscale<-1>(tmy - qxy);
    q = tdiv(T(f3), am);  split[3 * S + o] = tscale<-1>(te + q);   split[7 * S + o] = tscale<-1>(te - q);
    q = tdiv(T(my), am);  split[8 * S + o] = tscale<-1>(tr + q);   split[12 * S + o] = tscale<-1>(tr - q);
    split[9 * S + o] = tscale<-1>(tmx + qxy); split[13 * S + o] = tscale<-1>(tmx - qxy);
    q = tdiv(T(g2), am);  split[10 * S + o] = tscale<-1>(tmy + q); split[14 * S + o] = tscale<-1>(tmy - q);
    q = tdiv(T(g3), am);  split[11 * S + o] = tscale<-1>(te + q);  split[15 * S + o] = tscale<-1>(te - q);
  } else {
    if (which & 1) {
      // x segments whose local columns s*nxl-2 .. s*nxl+nxl+3 hold column i
      const int sh = min(p.cut_x - 1, (i + 2) / p.nxl);
      const int sl = i > 3 ? max(0, (i - 3 + p.nxl - 1) / p.nxl - 1) : 0;
      for (int sx = sl; sx <= sh; ++sx) {
        const T am = T(p.seg_ax[(int64_t)(j + 2) * p.cut_x + sx]);
        const int64_t os = seg_x_off(p, i, j, sx);
        T q;
        q = tdiv(T(mx), am);  split[0 * S + os] = tscale<-1>(tr + q);  split[4 * S + os] = tscale<-1>(tr - q);
        q = tdiv(T(f1), am);  split[1 * S + os] = tscale<-1>(tmx + q); split[5 * S + os] = tscale<-1>(tmx - q);
        q = tdiv(T(fxy), am); split[2 * S + os] = tscale<-1>(tmy + q); split[6 * S + os] = tscale<-1>(tmy - q);
        q = tdiv(T(f3), am);  split[3 * S + os] = tscale<-1>(te + q);  split[7 * S + os] = tscale<-1>(te - q);
      }
    }
    if (which & 2) {
      const int th = min(p.cut_y - 1, (j + 2) / p.nyl);
      const int tl = j > 3 ? max(0, (j - 3 + p.nyl - 1) / p.nyl - 1) : 0;
      for (int sy = tl; sy <= th; ++sy) {
        const T am = T(p.seg_ay[(int64_t)(i + 2) * p.cut_y + sy]);
        const int64_t os = seg_y_off(p, i, j, sy);
        double r2 = rho, m2 = mx, n2 = my, e2 = e, fxy2 = fxy, g22 = g2, g32 = g3;
        if (seg_sees_premirror(p, i, j, sy)) {  // this rank's ghost copy, pre-mirror
          const double* w = p.wall_save + ((int64_t)j * 3 + (p.total - i)) * 4;
          r2 = w[0];
          m2 = w[1];
          n2 = w[2];
          e2 = w[3];
          double ux = tdiv(m2, r2), uy = tdiv(n2, r2);
          if (p.flux_guard_eps2 ? (r2 < p.eps2) : (r2 < p.lim8_lt)) {
            ux = 0.;
            uy = 0.;
          }
          const double pr = g1 * (e2 - 0.5 * r2 * (ux * ux) - 0.5 * r2 * (uy * uy));
          fxy2 = r2 * ux * uy;
          g22 = r2 * (uy * uy) + pr;
          g32 = (e2 + pr) * uy;
        }
        const T tr2 = T(r2), tm2 = T(m2), tn2 = T(n2), te2 = T(e2);
        T q;
        q = tdiv(T(n2), am);   split[8 * S + os] = tscale<-1>(tr2 + q);  split[12 * S + os] = tscale<-1>(tr2 - q);
        q = tdiv(T(fxy2), am); split[9 * S + os] = tscale<-1>(tm2 + q);  split[13 * S + os] = tscale<-1>(tm2 - q);
        q = tdiv(T(g22), am);  split[10 * S + os] = tscale<-1>(tn2 + q); split[14 * S + os] = tscale<-1>(tn2 - q);
        q = tdiv(T(g32), am);  split[11 * S + os] = tscale<-1>(te2 + q); split[15 * S + os] = tscale<-1>(te2 - q);
      }
    }
  }
  // Roe preparation (x pass; the y pass is the same except in ex4 and ex6)
  if (which & 1) {
    double t0 = F32 ? ri : tdiv(1., rho);
    double vex = mx * t0, vey = my * t0;
    double pre = g1 * (e - tscale<-1>(mx * vex + my * vey));
    roe[0 * P + o] = sqrt_abs<T>(rho);
    roe[1 * P + o] = T(vex);
    roe[2 * P + o] = T(vey);
    roe[3 * P + o] = T((pre + e) * t0);
  }
  if (p.roe_reg_ex4 && (which & 2)) {
    // ex4_sedov_2d/main.f90:426
    double t0 = reg_recip(p, rho);
    double vex = mx * t0, vey = my * t0;
    double pre = g1 * (e - tscale<-1>(mx * vex + my * vey));
    roe[4 * P + o] = sqrt_abs<T>(rho);
    roe[5 * P + o] = T(vex);
    roe[6 * P + o] = T(vey);
    roe[7 * P + o] = T((pre + e) * t0);
  }
}

template <class T>
__global__ void k_prep2d(Params p, const double* __restrict__ u, const DevScalars* dsc,
                         T* __restrict__ split, T* __restrict__ roe, int which) {
  prep2d_cell<T>(p, u, dsc->alphamax, split, roe, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                 which);
}

template <class T>
__device__ __forceinline__ void prep1d_cell(const Params& p, const double* __restrict__ u,
                                            double amd, T* __restrict__ split, int t) {
  const Geom& g = p.g;
  if (t >= g.LI) return;
  const int64_t o = t, P = g.plane;
  T sp[3], sn[3];
  split1d<T>(p, ld(u + o), ld(u + P + o), ld(u + 2 * P + o), amd, sp, sn);
  for (int c = 0; c < 3; ++c) {
    split[c * P + o] = sp[c];
    split[(3 + c) * P + o] = sn[c];
  }
}

template <class T>
__global__ void k_prep1d(Params p, const double* __restrict__ u, const DevScalars* dsc,
                         T* __restrict__ split) {
  prep1d_cell<T>(p, u, dsc->alphamax, split, blockIdx.x * blockDim.x + threadIdx.x);
}

cudaError_t launch_prep(const Params& p, const double* u, const DevScalars* dsc, void* split,
                        void* roe, cudaStream_t s, int which) {
  const bool f32 = p.precision == SWFD_PRECISION_FP32_BULK;
  if (p.g.ndim == 1) {
    const int b = cell_block(p.g.LI), gb = (p.g.LI + b - 1) / b;
    if (f32) k_prep1d<float><<<gb, b, 0, s>>>(p, u, dsc, (float*)split);
    else k_prep1d<double><<<gb, b, 0, s>>>(p, u, dsc, (double*)split);
  } else {
    int64_t n = (int64_t)p.g.LI * p.g.LJ;
    const int b = cell_block(n, p.heavy_block);
    const unsigned gb = (unsigned)((n + b - 1) / b);
    if (f32) k_prep2d<float><<<gb, b, 0, s>>>(p, u, dsc, (float*)split, (float*)roe, which);
    else k_prep2d<double><<<gb, b, 0, s>>>(p, u, dsc, (double*)split, (double*)roe, which);
  }
  return cudaGetLastError();
}

// the work of wenofd before the interface fluxes: [ex6: alpha per rank row
// and column, x wall mirror] LF splitting + Roe preparation [ex6: y wall
// mirror, then the y pass's splitting]; *nk += kernels launched
cudaError_t launch_split(const Params& p, double* u, const DevScalars* dsc, void* split, void* roe,
                         cudaStream_t s, int* nk) {
  if (p.problem != SWFD_PROBLEM_SHOCK_DIFFRACTION) {
    *nk += 1;
    return launch_prep(p, u, dsc, split, roe, s, 3);
  }
  const int64_t ns = seg_alpha_items(p);
  k_seg_alpha<<<(unsigned)((ns + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(p);
  const int nwx = (min(6 * p.total, p.g.ny + 1) + 1) * 3, nwy = p.total * 3;
  k_wall_x<<<(nwx + 127) / 128, 128, 0, s>>>(p, u);
  cudaError_t e = launch_prep(p, u, dsc, split, roe, s, 1);
  if (e != cudaSuccess) return e;
  k_wall_y<<<(nwy + 127) / 128, 128, 0, s>>>(p, u);
  *nk += 5;
  return launch_prep(p, u, dsc, split, roe, s, 2);
}

// ---------------------------------------------------------------------------
// characteristic WENO5 flux of one interface (x: i+1/2 of row j; y: j+1/2 of
// column i).  sp/sn point at stencil cell -2, component 0 of the positive /
// negative split flux; components are P apart, stencil cells `step` apart.
// ---------------------------------------------------------------------------
// the eight binary64 reconstructions of one interface (four characteristic
// fields, both split fluxes) under a division policy (DivHw, DivFlag)
template <int YDIR, class D>
__device__ __forceinline__ void weno8_fp64(const Eigen2D<double>& E, const double* __restrict__ sp,
                                           const double* __restrict__ sn, int64_t P, int64_t step,
                                           double weps, D div, double* ur, double* ul) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double cp[5], cn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double* a = sp + m * step;
      const double* b = sn + m * step;
      const double a0 = ldt(a), a1 = ldt(a + P), a2 = ldt(a + 2 * P), a3 = ldt(a + 3 * P);
      const double b0 = ldt(b), b1 = ldt(b + P), b2 = ldt(b + 2 * P), b3 = ldt(b + 3 * P);
      if (k == 0) {
        cp[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, b0, b1, b2, b3);
      } else if (k == 1) {
        cp[m] = proj_row2<YDIR>(E.vt, a0, a1, a2);
        cn[m] = proj_row2<YDIR>(E.vt, b0, b1, b2);
      } else if (k == 2) {
        cp[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, b0, b1, b2, b3);
      } else {
        cp[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, b0, b1, b2, b3);
      }
    }
    ur[k] = weno_right(cp[0], cp[1], cp[2], cp[3], cp[4], weps, div);
    ul[k] = weno_left(cn[0], cn[1], cn[2], cn[3], cn[4], weps, div);
  }
}
struct Weno8 {
  double ur[4], ul[4];
};
// the rare interface whose divisions leave sd::div's own range: the same
// reconstructions with the exact fallback (out of line: the hot path stays
// free of the fallback branches)
template <int YDIR>
static __device__ __noinline__ Weno8 weno8_hw(Eigen2D<double> E, const double* sp,
                                              const double* sn, int64_t P, int64_t step,
                                              double weps) {
  Weno8 w;
  weno8_fp64<YDIR>(E, sp, sn, P, step, weps, DivHw(), w.ur, w.ul);
  return w;
}

// the eight binary32 reconstructions of one interface from its stencil
// values, [stencil cell][component] of the positive (a) and negative (b)
// split fluxes: each is projected onto the four characteristic fields and
// reconstructed (weno_right for a, weno_left for b)
template <int YDIR>
__device__ __forceinline__ void weno8_f32(const Eigen2D<float>& E, const float (&a)[5][4],
                                          const float (&b)[5][4], float weps, float ur[4],
                                          float ul[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float cp[5], cn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float *x = a[m], *y = b[m];
      if (k == 0) {
        cp[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, x[0], x[1], x[2], x[3]);
        cn[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, y[0], y[1], y[2], y[3]);
      } else if (k == 1) {
        cp[m] = proj_row2<YDIR>(E.vt, x[0], x[1], x[2]);
        cn[m] = proj_row2<YDIR>(E.vt, y[0], y[1], y[2]);
      } else if (k == 2) {
        cp[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, x[0], x[1], x[2], x[3]);
        cn[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, y[0], y[1], y[2], y[3]);
      } else {
        cp[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, x[0], x[1], x[2], x[3]);
        cn[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, y[0], y[1], y[2], y[3]);
      }
    }
    ur[k] = weno_right(cp[0], cp[1], cp[2], cp[3], cp[4], weps);
    ul[k] = weno_left(cn[0], cn[1], cn[2], cn[3], cn[4], weps);
  }
}

// evr . ur (main.f90:226-229): row 1 [1,0,1,1]; normal-momentum row
// [vn-c, 0, vn, vn+c]; tangential row [vt, 1, vt, vt]; energy row
// [H-vn c, vt, q, H+vn c]
template <int YDIR, class T>
__device__ __forceinline__ void back_project(const Eigen2D<T>& E, const T ur[4], const T ul[4],
                                             T outp[4], T outn[4]) {
  const int n = YDIR ? 2 : 1, tt = YDIR ? 1 : 2;
  if constexpr (sizeof(T) == 4) {  // FP32-bulk: fused multiply-adds
    outp[0] = ur[0] + ur[2] + ur[3];
    outn[0] = ul[0] + ul[2] + ul[3];
    outp[n] = fmaf(E.e_np, ur[3], fmaf(E.vn, ur[2], E.e_nm * ur[0]));
    outn[n] = fmaf(E.e_np, ul[3], fmaf(E.vn, ul[2], E.e_nm * ul[0]));
    outp[tt] = fmaf(E.vt, ur[3], fmaf(E.vt, ur[2], fmaf(E.vt, ur[0], ur[1])));
    outn[tt] = fmaf(E.vt, ul[3], fmaf(E.vt, ul[2], fmaf(E.vt, ul[0], ul[1])));
    outp[3] = fmaf(E.e_hp, ur[3], fmaf(E.qm, ur[2], fmaf(E.vt, ur[1], E.e_hm * ur[0])));
    outn[3] = fmaf(E.e_hp, ul[3], fmaf(E.qm, ul[2], fmaf(E.vt, ul[1], E.e_hm * ul[0])));
    return;
  }
  outp[0] = ur[0] + ur[2] + ur[3];
  outn[0] = ul[0] + ul[2] + ul[3];
  outp[n] = E.e_nm * ur[0] + E.vn * ur[2] + E.e_np * ur[3];
  outn[n] = E.e_nm * ul[0] + E.vn * ul[2] + E.e_np * ul[3];
  outp[tt] = E.vt * ur[0] + ur[1] + E.vt * ur[2] + E.vt * ur[3];
  outn[tt] = E.vt * ul[0] + ul[1] + E.vt * ul[2] + E.vt * ul[3];
  outp[3] = E.e_hm * ur[0] + E.vt * ur[1] + E.qm * ur[2] + E.e_hp * ur[3];
  outn[3] = E.e_hm * ul[0] + E.vt * ul[1] + E.qm * ul[2] + E.e_hp * ul[3];
}

template <int YDIR, class T, bool QD = false>
__device__ __forceinline__ void interface_flux(const Eigen2D<T>& E, const T* __restrict__ sp,
                                               const T* __restrict__ sn, int64_t P, int64_t step,
                                               T weps, T outp[4], T outn[4],
                                               const QuadWeno* qw = nullptr) {
  T ur[4], ul[4];
  if constexpr (sizeof(T) == 4) {
    // FP32: the 5 x 4 stencil values of each split flux are loaded once into
    // registers (40 loads instead of 160 per interface) and projected from
    // there; the arithmetic is the same as below
    T a[5][4], b[5][4];
#pragma unroll
    for (int m = 0; m < 5; ++m)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        a[m][c] = ldt(sp + m * step + c * P);
        b[m][c] = ldt(sn + m * step + c * P);
      }
    weno8_f32<YDIR>(E, a, b, weps, ur, ul);
  } else if constexpr (!QD) {
    // every division without its fallback branch; one check for all eight
    int bad = 0;
    weno8_fp64<YDIR>(E, sp, sn, P, step, weps, DivFlag{&bad}, ur, ul);
    if (bad) {
      const Weno8 w = weno8_hw<YDIR>(E, sp, sn, P, step, weps);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ur[k] = w.ur[k];
        ul[k] = w.ul[k];
      }
    }
  } else
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T cp[5], cn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const T* a = sp + m * step;
      const T* b = sn + m * step;
      T a0 = ldt(a), a1 = ldt(a + P), a2 = ldt(a + 2 * P), a3 = ldt(a + 3 * P);
      T b0 = ldt(b), b1 = ldt(b + P), b2 = ldt(b + 2 * P), b3 = ldt(b + 3 * P);
      if (k == 0) {
        cp[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, b0, b1, b2, b3);
      } else if (k == 1) {
        cp[m] = proj_row2<YDIR>(E.vt, a0, a1, a2);
        cn[m] = proj_row2<YDIR>(E.vt, b0, b1, b2);
      } else if (k == 2) {
        cp[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, b0, b1, b2, b3);
      } else {
        cp[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, a0, a1, a2, a3);
        cn[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, b0, b1, b2, b3);
      }
    }
    ur[k] = weno_right_qd(cp[0], cp[1], cp[2], cp[3], cp[4], *qw);
    ul[k] = weno_left_qd(cn[0], cn[1], cn[2], cn[3], cn[4], *qw);
  }
  back_project<YDIR, T>(E, ur, ul, outp, outn);
}

// 1D: eigenvectors at cell m (ex2_sedov_1d/main.f90:89-157); vxm and hm come
// from the FP64 state (pressure recovery), the rest is in T
template <class T, bool QD = false>
__device__ __forceinline__ void flux1d_lane(const Params& p, const double* __restrict__ u,
                                            const T* __restrict__ split, T* __restrict__ flux,
                                            int t, unsigned long long* cnt) {
  // eight lanes per cell: lanes 0..5 of a group each reconstruct one
  // characteristic field (k = lane / 2) of one side (lane % 2: the positive
  // flux at the right face, the negative one), so that the six WENO chains of
  // a cell run side by side instead of one after another in one thread (a
  // tiny 1D grid leaves the FP64 pipes idle and its time is the length of
  // these dependent chains); the group then exchanges the six values and
  // lanes 0..5 form the six output components.  Every value is computed by
  // the same expression as in a one-thread-per-cell form.
  // t: the lane's index; lanes 8m..8m+7 are lanes of one warp (the group's
  // shuffles), and every lane of the warp takes part
  const Geom& g = p.g;
  const int m = t >> 3, sub = t & 7;  // cell 0..n+1, lane in its group
  const bool active = m <= g.nx + 1;
  const int mm = active ? m : g.nx + 1;  // inactive lanes repeat the last cell
  const int64_t P = g.plane, o = g.at(mm, -2);
  Eigen1D<T> E;
  eigen1d<T>(p.gamma1, ld(u + o), ld(u + P + o), ld(u + 2 * P + o), E);
  const T v = recon1d<T, QD>(p, E, sub, [&](int side, int c, int jj) {
    return ldt(split + (side ? 3 * P : 0) + c * P + o + jj - 2);
  });
  const T r = back1d<T>(E, v, sub);
  if (!p.limiter) {
    if (active && sub < 6) flux[sub * P + o] = r;
    return;
  }
  // use_limiter 1: lanes 0 and 3 limit and store their side's components
  T w[3];
  int nd = 0, np = 0;
  const bool lim = limit1d_group<T>(
      p, r, sub, [&](int side, int c) { return ldt(split + (side ? 3 * P : 0) + c * P + o); }, w,
      nd, np);
  if (active && lim) {
#pragma unroll
    for (int c = 0; c < 3; ++c) flux[(sub + c) * P + o] = w[c];
    count_limited(cnt, nd, np);
  }
}

template <class T, bool QD = false>
__global__ void k_flux1d(Params p, const double* __restrict__ u, const T* __restrict__ split,
                         T* __restrict__ flux, unsigned long long* cnt) {
  flux1d_lane<T, QD>(p, u, split, flux, blockIdx.x * blockDim.x + threadIdx.x, cnt);
}

// Both directions in one persistent launch: a grid of exactly the resident
// blocks, whose warps take chunks of 32 consecutive interfaces (x interfaces
// of rows 1..ny first, then y interfaces of rows 0..ny+1) from a counter, so
// the pipes stay busy to the last chunk instead of idling through the tail of
// a partial last wave.
#define SWFD_FLUX_BLOCK 128
// resident blocks per SM: the FP64 pipe saturates with 3 (168 registers);
// the FP32 pipe needs more warps in flight
#define SWFD_FLUX_MINB(T) (sizeof(T) == 8 ? 3 : 4)
// use_limiter = 1: the positivity limiter of one split flux at its interface
// (ex3_vortex_accuracy_2d/main.f90:241-329, y pass :444-530; ex6 clamps theta
// at 0, ex6_shock_diffraction/main.f90:330,351,379,398).  sp: the split flux
// of the interface's left cell (components S apart), out: its reconstructed
// flux, limited in place; nd, np count the density and pressure limitings.
template <class T>
__device__ __forceinline__ void zs_limit(const Params& p, const T* __restrict__ sp, int64_t S,
                                         T out[4], int& nd, int& np) {
  const T g1 = T(p.gamma1);
  const T d_ave = ldt(sp), m_ave = ldt(sp + S), n_ave = ldt(sp + 2 * S), e_ave = ldt(sp + 3 * S);
  const T ave[4] = {d_ave, m_ave, n_ave, e_ave};
  const T p_ave = g1 * (e_ave - T(0.5) * (m_ave * m_ave) / d_ave - T(0.5) * (n_ave * n_ave) / d_ave);
  T pt[2][4];
  for (int c = 0; c < 4; ++c) {
    pt[0][c] = out[c];
    pt[1][c] = (ave[c] - out[c] / T(12.)) / T(11. / 12.);
  }
  T theta = T(1.);
  for (int ig = 0; ig < 2; ++ig) {
    const T d_l = pt[ig][0];
    if (d_l < T(0.)) theta = fmin(theta, fabs(d_ave - T(0.)) / fabs(d_ave - d_l));
  }
  if (p.limiter_clamp) theta = fmax(theta, T(0.));
  if (theta < T(1.)) {
    out[0] = theta * out[0] + (T(1.) - theta) * d_ave;
    ++nd;
  }
  theta = T(1.);
  pt[0][0] = out[0];
  pt[1][0] = (ave[0] - out[0] / T(12.)) / T(11. / 12.);
  for (int ig = 0; ig < 2; ++ig) {
    const T d_l = pt[ig][0], m_l = pt[ig][1], n_l = pt[ig][2], e_l = pt[ig][3];
    const T p_l = g1 * (e_l - (m_l * m_l) / d_l / T(2.) - (n_l * n_l) / d_l / T(2.));
    if (p_l < T(0.)) theta = fmin(theta, fabs(p_ave - T(0.)) / fabs(p_ave - p_l));
  }
  if (p.limiter_clamp) theta = fmax(theta, T(0.));
  if (theta < T(1.)) {
    ++np;
    for (int c = 0; c < 4; ++c) out[c] = theta * out[c] + (T(1.) - theta) * ave[c];
  }
}


// the 32 interfaces of chunk c (x chunks first, then y chunks).  SEG: the
// problem may have rank segments (ex6); without them the face index maps
// directly to the cell offset.
// per-launch constants of the flux kernel, converted to T once
template <class T>
struct FluxConst {
  T g1, weps;
};
template <class T>
__device__ __forceinline__ FluxConst<T> flux_const(const Params& p) {
  return FluxConst<T>{T(p.gamma1), T(p.weno_eps)};
}

template <class T, bool SEG, bool LIM = false, bool QD = false>
__device__ __forceinline__ void flux_chunk(const Params& p, const T* __restrict__ split,
                                           const T* __restrict__ roe, T am, T* __restrict__ flux,
                                           int64_t c, int64_t chunks_x, int lane,
                                           unsigned long long* cnt, const FluxConst<T>& cst) {
  const Geom& g = p.g;
  const int64_t P = g.plane, pit = g.pitch, S = p.sg.plane, spit = p.sg.pitch;
  const T g1 = cst.g1, weps = cst.weps;
  QuadWeno qw;
  const qd::q128* qreg = nullptr;
  if constexpr (QD) {
    qw.c1312 = p.q_c1312;
    qw.eps = p.q_weno_eps;
    if (p.roe_reg_ex4) qreg = &p.q_1em15;
  }
  {
    T op[4], on[4];
    if (c < chunks_x) {
      int64_t t = (int64_t)c * 32 + lane;
      if (t >= flux_faces_x(p, LIM)) return;
      const int lsx = p.nxl + 2, lx = p.cut_x * lsx;
      const int r = ((int)t % lx), rr = ((int)t / lx);
      const int j = LIM ? (rr / (p.nyl + 2)) * p.nyl + rr % (p.nyl + 2) : rr + 1;
      const int sx = SEG ? r / lsx : 0, i = SEG ? sx * p.nxl + r % lsx : r;
      const int64_t o = g.at(i, j), os = SEG ? seg_x_off(p, i, j, sx) : o;
      if (SEG && p.seg_alpha) am = T(p.seg_ax[(int64_t)(j + 2) * p.cut_x + sx]);
      Eigen2D<T> E;
      roe_eigen2d<T, QD>(g1, 0, ldt(roe + o), ldt(roe + o + 1), ldt(roe + P + o),
                     ldt(roe + P + o + 1), ldt(roe + 2 * P + o), ldt(roe + 2 * P + o + 1),
                     ldt(roe + 3 * P + o), ldt(roe + 3 * P + o + 1), E, qreg);
      interface_flux<0, T, QD>(E, split + os - 2, split + 4 * S + os - 2, S, 1, weps, op, on,
                               &qw);
      if (LIM) {
        int nd = 0, np = 0;
        zs_limit<T>(p, split + os, S, op, nd, np);
        zs_limit<T>(p, split + 4 * S + os, S, on, nd, np);
        count_limited(cnt, nd, np);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        flux[k * S + os] = p.alpha_premul ? am * op[k] : op[k];
        flux[(4 + k) * S + os] = p.alpha_premul ? am * on[k] : on[k];
      }
    } else {
      int64_t t = (int64_t)(c - chunks_x) * 32 + lane;
      if (t >= flux_faces_y(p, LIM)) return;
      const int lsy = p.nyl + 2;
      const int ncol = (int)flux_cols_y(p, LIM), ci = ((int)t % ncol), r = ((int)t / ncol);
      const int i = LIM ? (ci / (p.nxl + 2)) * p.nxl + ci % (p.nxl + 2) : ci + 1;
      const int sy = SEG ? r / lsy : 0, j = SEG ? sy * p.nyl + r % lsy : r;
      const int64_t o = g.at(i, j), os = SEG ? seg_y_off(p, i, j, sy) : o;
      if (SEG && p.seg_alpha) am = T(p.seg_ay[(int64_t)(i + 2) * p.cut_y + sy]);
      const T* rr = roe + (p.roe_reg_ex4 ? 4 * P : 0);
      T wr = ldt(rr + o + pit), vxr = ldt(rr + P + o + pit), vyr = ldt(rr + 2 * P + o + pit),
        hr = ldt(rr + 3 * P + o + pit);
      if (SEG && seg_sees_premirror(p, i, j + 1, sy)) {
        // the ex6 rank's ghost row j+1 (local nyl+2), pre-mirror, with the
        // y pass's preparation (ex4_sedov_2d/main.f90:426)
        const double* w = p.wall_save + ((int64_t)(j + 1) * 3 + (p.total - i)) * 4;
        double t0;
        if constexpr (QD) t0 = reg_recip(p, w[0]);
        else t0 = 1. / (w[0] + 1e-15);
        const double vex = w[1] * t0, vey = w[2] * t0;
        const double pre = p.gamma1 * (w[3] - 0.5 * (w[1] * vex + w[2] * vey));
        wr = sqrt_abs<T>(w[0]);
        vxr = T(vex);
        vyr = T(vey);
        hr = T((pre + w[3]) * t0);
      }
      Eigen2D<T> E;
      roe_eigen2d<T, QD>(g1, 1, ldt(rr + o), wr, ldt(rr + P + o), vxr, ldt(rr + 2 * P + o), vyr,
                     ldt(rr + 3 * P + o), hr, E, qreg);
      interface_flux<1, T, QD>(E, split + 8 * S + os - 2 * spit, split + 12 * S + os - 2 * spit,
                               S, spit, weps, op, on, &qw);
      if (LIM) {
        int nd = 0, np = 0;
        zs_limit<T>(p, split + 8 * S + os, S, op, nd, np);
        zs_limit<T>(p, split + 12 * S + os, S, on, nd, np);
        count_limited(cnt, nd, np);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        flux[(8 + k) * S + os] = p.alpha_premul ? am * op[k] : op[k];
        flux[(12 + k) * S + os] = p.alpha_premul ? am * on[k] : on[k];
      }
    }
  }
}

template <class T, bool SEG, bool LIM, int MINB = SWFD_FLUX_MINB(T), bool QD = false>
__global__ void __launch_bounds__(SWFD_FLUX_BLOCK, MINB)
    k_flux_xy(Params p, const T* __restrict__ split, const T* __restrict__ roe,
              const DevScalars* dsc, T* __restrict__ flux, int* __restrict__ work) {
  const int64_t chunks_x = (flux_faces_x(p, LIM) + 31) / 32;
  const int64_t chunks = chunks_x + (flux_faces_y(p, LIM) + 31) / 32;
  const int lane = threadIdx.x & 31;
  const T am = p.alpha_premul ? T(dsc->alphamax) : T(1.0);
  const FluxConst<T> cst = flux_const<T>(p);
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= chunks) break;
    flux_chunk<T, SEG, LIM, QD>(p, split, roe, am, flux, c, chunks_x, lane,
                            (unsigned long long*)&dsc->den_count, cst);
  }
  // work[1] counts the warps that found the chunks exhausted: the last one
  // out re-arms both counters for the next launch (every other warp's final
  // fetch precedes its increment of work[1])
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(work + 1, 1) == (int)(gridDim.x * (blockDim.x >> 5)) - 1) {
      atomicExch(work, 0);
      atomicExch(work + 1, 0);
    }
  }
}

// ---------------------------------------------------------------------------
// FP64 interface fluxes with two lanes per interface (no rank segments, no
// limiter, binary64 literals): lane 0 of a pair reconstructs the positive
// split flux (four weno_right, its back projection), lane 1 the negative one
// (four weno_left); both form the interface's Roe eigenvectors.  Each lane
// holds half the stencil values and chains of one side, so more warps fit an
// SM and each has shorter dependent chains, at the price of the eigenvectors
// computed twice.  Every value is the one-lane form's expression.
// ---------------------------------------------------------------------------
template <int YDIR, class D>
__device__ __forceinline__ void weno4_side(const Eigen2D<double>& E, const double* __restrict__ s,
                                           int64_t P, int64_t step, double weps, int side, D div,
                                           double out[4]) {
  const int n = YDIR ? 2 : 1, tt = YDIR ? 1 : 2;
  double w[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    double c[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double* a = s + m * step;
      const double a0 = ldt(a), a1 = ldt(a + P), a2 = ldt(a + 2 * P), a3 = ldt(a + 3 * P);
      if (k == 0) c[m] = proj_row<YDIR>(E.l1_0, E.l1_n, E.l1_t, E.l1_3, a0, a1, a2, a3);
      else if (k == 1) c[m] = proj_row2<YDIR>(E.vt, a0, a1, a2);
      else if (k == 2) c[m] = proj_row<YDIR>(E.l3_0, E.l3_n, E.l3_t, E.l3_3, a0, a1, a2, a3);
      else c[m] = proj_row<YDIR>(E.l4_0, E.l4_n, E.l4_t, E.l4_3, a0, a1, a2, a3);
    }
    w[k] = weno_side(c[0], c[1], c[2], c[3], c[4], side, weps, div);
  }
  // evr . w (as interface_flux's back projection)
  out[0] = w[0] + w[2] + w[3];
  out[n] = E.e_nm * w[0] + E.vn * w[2] + E.e_np * w[3];
  out[tt] = E.vt * w[0] + w[1] + E.vt * w[2] + E.vt * w[3];
  out[3] = E.e_hm * w[0] + E.vt * w[1] + E.qm * w[2] + E.e_hp * w[3];
}
struct Side4 {
  double v[4];
};
template <int YDIR>
static __device__ __noinline__ Side4 weno4_side_hw(Eigen2D<double> E, const double* s, int64_t P,
                                                   int64_t step, double weps, int side) {
  Side4 r;
  weno4_side<YDIR>(E, s, P, step, weps, side, DivHw(), r.v);
  return r;
}
template <int YDIR>
__device__ __forceinline__ void side_flux(const Eigen2D<double>& E, const double* s, int64_t P,
                                          int64_t step, double weps, int side, double out[4]) {
  int bad = 0;
  weno4_side<YDIR>(E, s, P, step, weps, side, DivFlag{&bad}, out);
  if (bad) {
    const Side4 r = weno4_side_hw<YDIR>(E, s, P, step, weps, side);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = r.v[k];
  }
}

// 16 interfaces of chunk c (x chunks first, then y chunks), two lanes each
__device__ __forceinline__ void flux_chunk_pair(const Params& p, const double* __restrict__ split,
                                                const double* __restrict__ roe, double am,
                                                double* __restrict__ flux, int64_t c,
                                                int64_t chunks_x, int lane) {
  const Geom& g = p.g;
  const int64_t P = g.plane, pit = g.pitch, S = p.sg.plane, spit = p.sg.pitch;
  const double g1 = p.gamma1, weps = p.weno_eps;
  const int side = lane & 1;
  double o4[4];
  if (c < chunks_x) {
    const int64_t t = c * 16 + (lane >> 1);
    if (t >= flux_faces_x(p)) return;
    const int lx = p.nxl + 2;  // faces i = 0..nx+1 of rows 1..ny (one segment)
    const int i = (int)t % lx, j = (int)t / lx + 1;
    const int64_t o = g.at(i, j);
    Eigen2D<double> E;
    roe_eigen2d<double>(g1, 0, ldt(roe + o), ldt(roe + o + 1), ldt(roe + P + o),
                        ldt(roe + P + o + 1), ldt(roe + 2 * P + o), ldt(roe + 2 * P + o + 1),
                        ldt(roe + 3 * P + o), ldt(roe + 3 * P + o + 1), E);
    side_flux<0>(E, split + 4 * side * S + o - 2, S, 1, weps, side, o4);
#pragma unroll
    for (int k = 0; k < 4; ++k) flux[(4 * side + k) * S + o] = p.alpha_premul ? am * o4[k] : o4[k];
  } else {
    const int64_t t = (c - chunks_x) * 16 + (lane >> 1);
    if (t >= flux_faces_y(p)) return;
    const int i = (int)t % g.nx + 1, j = (int)t / g.nx;
    const int64_t o = g.at(i, j);
    const double* rr = roe + (p.roe_reg_ex4 ? 4 * P : 0);
    Eigen2D<double> E;
    roe_eigen2d<double>(g1, 1, ldt(rr + o), ldt(rr + o + pit), ldt(rr + P + o),
                        ldt(rr + P + o + pit), ldt(rr + 2 * P + o), ldt(rr + 2 * P + o + pit),
                        ldt(rr + 3 * P + o), ldt(rr + 3 * P + o + pit), E);
    side_flux<1>(E, split + (8 + 4 * side) * S + o - 2 * spit, S, spit, weps, side, o4);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      flux[(8 + 4 * side + k) * S + o] = p.alpha_premul ? am * o4[k] : o4[k];
  }
}

template <int MINB>
__global__ void __launch_bounds__(SWFD_FLUX_BLOCK, MINB)
    k_flux_xy_pair(Params p, const double* __restrict__ split, const double* __restrict__ roe,
                   const DevScalars* dsc, double* __restrict__ flux, int* __restrict__ work) {
  const int64_t chunks_x = (flux_faces_x(p) + 15) / 16;
  const int64_t chunks = chunks_x + (flux_faces_y(p) + 15) / 16;
  const int lane = threadIdx.x & 31;
  const double am = p.alpha_premul ? dsc->alphamax : 1.0;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= chunks) break;
    flux_chunk_pair(p, split, roe, am, flux, c, chunks_x, lane);
  }
  if (lane == 0) {  // as k_flux_xy: the last warp out re-arms both counters
    __threadfence();
    if (atomicAdd(work + 1, 1) == (int)(gridDim.x * (blockDim.x >> 5)) - 1) {
      atomicExch(work, 0);
      atomicExch(work + 1, 0);
    }
  }
}

template <int MINB>
static int flux_grid_pair() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_flux_xy_pair<MINB>, SWFD_FLUX_BLOCK, 0);
    grid = sms * (per > 0 ? per : 1);
  }
  return grid;
}

// ---------------------------------------------------------------------------
// The lane-pair interface fluxes as one short instruction stream: the x and y
// interfaces share one code path (the direction is warp-uniform: a chunk holds
// interfaces of one direction; it selects the addresses, the projection
// coefficients' order and the output planes), and one reconstruction runs in
// a loop over the four characteristic fields, the back projection accumulated
// field by field in the order of its sums.  Every value is the lane-pair
// kernel's expression; the code a warp executes per interface is about an
// eighth of the unrolled form's, which the instruction cache holds while 16
// warps per SM are at different points of it.
// ---------------------------------------------------------------------------
template <class D>
__device__ __forceinline__ void weno4_side_loop(const Eigen2D<double>& E, int ydir,
                                                const double* __restrict__ s, int64_t P,
                                                int64_t step, double weps, int side, D div,
                                                double& o0, double& on, double& ot, double& o3) {
  const double nvt = tneg(E.vt);
#pragma unroll 1
  for (int k = 0; k < 4; ++k) {
    double c[5];
    if (k == 1) {  // evl row 2: x pass -vt*f0 + f2, y pass -vt*f0 + f1
      const int64_t pg = ydir ? P : 2 * P;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double* a = s + m * step;
        c[m] = nvt * ldt(a) + ldt(a + pg);
      }
    } else {
      // rows 1, 3, 4: l0*f0 + ln*f1 + lt*f2 + l3*f3 (x), l0*f0 + lt*f1 + ln*f2 + l3*f3 (y)
      const double l0 = k == 0 ? E.l1_0 : k == 2 ? E.l3_0 : E.l4_0;
      const double ln = k == 0 ? E.l1_n : k == 2 ? E.l3_n : E.l4_n;
      const double lt = k == 0 ? E.l1_t : k == 2 ? E.l3_t : E.l4_t;
      const double l3 = k == 0 ? E.l1_3 : k == 2 ? E.l3_3 : E.l4_3;
      const double k1 = ydir ? lt : ln, k2 = ydir ? ln : lt;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double* a = s + m * step;
        c[m] = l0 * ldt(a) + k1 * ldt(a + P) + k2 * ldt(a + 2 * P) + l3 * ldt(a + 3 * P);
      }
    }
    const double w = weno_side(c[0], c[1], c[2], c[3], c[4], side, weps, div);
    // evr . w, each sum in its order:
    //   o0 = w0 + w2 + w3,  on = e_nm w0 + vn w2 + e_np w3,
    //   ot = vt w0 + w1 + vt w2 + vt w3,  o3 = e_hm w0 + vt w1 + qm w2 + e_hp w3
    if (k == 0) {
      o0 = w;
      on = E.e_nm * w;
      ot = E.vt * w;
      o3 = E.e_hm * w;
    } else if (k == 1) {
      ot = ot + w;
      o3 = o3 + E.vt * w;
    } else {
      const double cn = k == 2 ? E.vn : E.e_np, c3 = k == 2 ? E.qm : E.e_hp;
      o0 = o0 + w;
      on = on + cn * w;
      ot = ot + E.vt * w;
      o3 = o3 + c3 * w;
    }
  }
}
static __device__ __noinline__ Side4 weno4_side_loop_hw(Eigen2D<double> E, int ydir,
                                                        const double* s, int64_t P, int64_t step,
                                                        double weps, int side) {
  Side4 r;
  weno4_side_loop(E, ydir, s, P, step, weps, side, DivHw(), r.v[0], r.v[1], r.v[2], r.v[3]);
  return r;
}

template <int MINB>
__global__ void __launch_bounds__(SWFD_FLUX_BLOCK, MINB)
    k_flux_xy_loop(Params p, const double* __restrict__ split, const double* __restrict__ roe,
                   const DevScalars* dsc, double* __restrict__ flux, int* __restrict__ work) {
  const Geom& g = p.g;
  const int64_t chunks_x = (flux_faces_x(p) + 15) / 16;
  const int64_t chunks = chunks_x + (flux_faces_y(p) + 15) / 16;
  const int lane = threadIdx.x & 31, side = lane & 1;
  const double am = p.alpha_premul ? dsc->alphamax : 1.0;
  const int64_t P = g.plane, S = p.sg.plane, spit = p.sg.pitch;
  const double g1 = p.gamma1, weps = p.weno_eps;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= chunks) break;
    // the interface: its direction, offset, Roe neighbour, stencil start and step
    int ydir;
    int64_t o, rnb, step;
    const double* rb;
    if (c < chunks_x) {
      const int64_t t = (int64_t)c * 16 + (lane >> 1);
      if (t >= flux_faces_x(p)) continue;
      const int lx = p.nxl + 2;  // faces i = 0..nx+1 of rows 1..ny (one segment)
      o = g.at((int)t % lx, (int)t / lx + 1);
      ydir = 0, rnb = 1, step = 1, rb = roe;
    } else {
      const int64_t t = ((int64_t)c - chunks_x) * 16 + (lane >> 1);
      if (t >= flux_faces_y(p)) continue;
      o = g.at((int)t % g.nx + 1, (int)t / g.nx);
      ydir = 1, rnb = g.pitch, step = spit, rb = roe + (p.roe_reg_ex4 ? 4 * P : 0);
    }
    Eigen2D<double> E;
    roe_eigen2d<double>(g1, ydir, ldt(rb + o), ldt(rb + o + rnb), ldt(rb + P + o),
                        ldt(rb + P + o + rnb), ldt(rb + 2 * P + o), ldt(rb + 2 * P + o + rnb),
                        ldt(rb + 3 * P + o), ldt(rb + 3 * P + o + rnb), E);
    const int64_t pl = 8 * ydir + 4 * side;  // the side's first split and flux plane
    const double* s = split + pl * S + o - 2 * step;
    double o0, on, ot, o3;
    int bad = 0;
    weno4_side_loop(E, ydir, s, S, step, weps, side, DivFlag{&bad}, o0, on, ot, o3);
    if (bad) {
      const Side4 r = weno4_side_loop_hw(E, ydir, s, S, step, weps, side);
      o0 = r.v[0], on = r.v[1], ot = r.v[2], o3 = r.v[3];
    }
    double* f = flux + pl * S + o;
    const int64_t fn = ydir ? 2 * S : S, ft = ydir ? S : 2 * S;
    f[0] = p.alpha_premul ? am * o0 : o0;
    f[fn] = p.alpha_premul ? am * on : on;
    f[ft] = p.alpha_premul ? am * ot : ot;
    f[3 * S] = p.alpha_premul ? am * o3 : o3;
  }
  if (lane == 0) {  // as k_flux_xy: the last warp out re-arms both counters
    __threadfence();
    if (atomicAdd(work + 1, 1) == (int)(gridDim.x * (blockDim.x >> 5)) - 1) {
      atomicExch(work, 0);
      atomicExch(work + 1, 0);
    }
  }
}

// The short lane-pair kernel with each interface's eigenvectors formed once:
// a warp takes 32 interfaces of one direction, each lane forms one
// interface's Roe eigenvectors into shared memory, then the lane pairs
// reconstruct the interfaces in two rounds of 16 (lane 0 of a pair the
// positive split flux, lane 1 the negative one), reading the eigenvectors
// back.  About 40 FP64 instructions fewer per interface than forming them
// in both lanes; every value is k_flux_xy_loop's.
constexpr int EIG2D_N = 19;  // the Eigen2D entries the reconstruction uses
__device__ __forceinline__ void eig2d_store(const Eigen2D<double>& E, double* s) {
  const double v[EIG2D_N] = {E.vn,   E.vt,   E.qm,   E.e_nm, E.e_np, E.e_hm, E.e_hp,
                             E.l1_0, E.l1_n, E.l1_t, E.l1_3, E.l3_0, E.l3_n, E.l3_t,
                             E.l3_3, E.l4_0, E.l4_n, E.l4_t, E.l4_3};
#pragma unroll
  for (int k = 0; k < EIG2D_N; ++k) s[32 * k] = v[k];
}
__device__ __forceinline__ void eig2d_load(Eigen2D<double>& E, const double* s) {
  double v[EIG2D_N];
#pragma unroll
  for (int k = 0; k < EIG2D_N; ++k) v[k] = s[32 * k];
  E.vn = v[0], E.vt = v[1], E.qm = v[2], E.e_nm = v[3], E.e_np = v[4], E.e_hm = v[5];
  E.e_hp = v[6], E.l1_0 = v[7], E.l1_n = v[8], E.l1_t = v[9], E.l1_3 = v[10];
  E.l3_0 = v[11], E.l3_n = v[12], E.l3_t = v[13], E.l3_3 = v[14], E.l4_0 = v[15];
  E.l4_n = v[16], E.l4_t = v[17], E.l4_3 = v[18];
  E.cm = 0.0;  // not used by the reconstruction
}

template <int MINB>
__global__ void __launch_bounds__(SWFD_FLUX_BLOCK, MINB)
    k_flux_xy_share(Params p, const double* __restrict__ split, const double* __restrict__ roe,
                    const DevScalars* dsc, double* __restrict__ flux, int* __restrict__ work) {
  __shared__ double sE[SWFD_FLUX_BLOCK / 32][EIG2D_N * 32];
  const Geom& g = p.g;
  const int64_t fx = flux_faces_x(p), fy = flux_faces_y(p);
  const int64_t chunks_x = (fx + 31) / 32;
  const int64_t chunks = chunks_x + (fy + 31) / 32;
  const int lane = threadIdx.x & 31, side = lane & 1;
  double* se = sE[threadIdx.x >> 5];
  const double am = p.alpha_premul ? dsc->alphamax : 1.0;
  const int64_t P = g.plane, S = p.sg.plane, spit = p.sg.pitch;
  const double g1 = p.gamma1, weps = p.weno_eps;
  const int lx = p.nxl + 2;  // x faces i = 0..nx+1 of rows 1..ny (one segment)
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= chunks) break;
    // 32 interfaces of one direction: t0 .. t0 + 31
    const int ydir = c < chunks_x ? 0 : 1;
    const int64_t t0 = ydir ? ((int64_t)c - chunks_x) * 32 : (int64_t)c * 32;
    const int64_t nfaces = ydir ? fy : fx;
    const int64_t rnb = ydir ? g.pitch : 1, step = ydir ? spit : 1;
    const double* rb = ydir ? roe + (p.roe_reg_ex4 ? 4 * P : 0) : roe;
    auto offset = [&](int64_t t) {
      return ydir ? g.at((int)t % g.nx + 1, (int)t / g.nx) : g.at((int)t % lx, (int)t / lx + 1);
    };
    {  // the eigenvectors of interface t0 + lane
      const int64_t t = t0 + lane;
      if (t < nfaces) {
        const int64_t o = offset(t);
        Eigen2D<double> E;
        roe_eigen2d<double>(g1, ydir, ldt(rb + o), ldt(rb + o + rnb), ldt(rb + P + o),
                            ldt(rb + P + o + rnb), ldt(rb + 2 * P + o),
                            ldt(rb + 2 * P + o + rnb), ldt(rb + 3 * P + o),
                            ldt(rb + 3 * P + o + rnb), E);
        eig2d_store(E, se + lane);
      }
    }
    __syncwarp();
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {  // interfaces t0 + 16 h + lane / 2, two lanes each
      const int j = 16 * h + (lane >> 1);
      const int64_t t = t0 + j;
      if (t < nfaces) {
        const int64_t o = offset(t);
        Eigen2D<double> E;
        eig2d_load(E, se + j);
        const int64_t pl = 8 * ydir + 4 * side;  // the side's first split and flux plane
        const double* s = split + pl * S + o - 2 * step;
        double o0, on, ot, o3;
        int bad = 0;
        weno4_side_loop(E, ydir, s, S, step, weps, side, DivFlag{&bad}, o0, on, ot, o3);
        if (bad) {
          const Side4 r = weno4_side_loop_hw(E, ydir, s, S, step, weps, side);
          o0 = r.v[0], on = r.v[1], ot = r.v[2], o3 = r.v[3];
        }
        double* f = flux + pl * S + o;
        const int64_t fn = ydir ? 2 * S : S, ft = ydir ? S : 2 * S;
        f[0] = p.alpha_premul ? am * o0 : o0;
        f[fn] = p.alpha_premul ? am * on : on;
        f[ft] = p.alpha_premul ? am * ot : ot;
        f[3 * S] = p.alpha_premul ? am * o3 : o3;
      }
    }
    __syncwarp();  // the next chunk rewrites se
  }
  if (lane == 0) {  // as k_flux_xy: the last warp out re-arms both counters
    __threadfence();
    if (atomicAdd(work + 1, 1) == (int)(gridDim.x * (blockDim.x >> 5)) - 1) {
      atomicExch(work, 0);
      atomicExch(work + 1, 0);
    }
  }
}

template <int MINB>
static int flux_grid_share() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_flux_xy_share<MINB>, SWFD_FLUX_BLOCK, 0);
    grid = sms * (per > 0 ? per : 1);
  }
  return grid;
}

template <int MINB>
static int flux_grid_loop() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_flux_xy_loop<MINB>, SWFD_FLUX_BLOCK, 0);
    grid = sms * (per > 0 ? per : 1);
  }
  return grid;
}

template <class T, int MINB = SWFD_FLUX_MINB(T)>
static int flux_grid() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_flux_xy<T, false, false, MINB>,
                                                  SWFD_FLUX_BLOCK, 0);
    grid = sms * (per > 0 ? per : 1);
  }
  return grid;
}

// Launch-shape variants of the common flux kernel (no rank segments, no
// limiter) that swfd_autotune times: resident blocks per SM, traded against
// registers per thread (FP64 one-lane kernel: 3 = 168 registers, 2 = 236, 4 =
// 128 with spills; FP32: 4 = 128, 5 = 102, 6 = 85), and for FP64 the
// lane-pair kernels.  The first entry is the default.
int flux_min_blocks_candidates(bool f32, int* out) {
  if (f32) {
    out[0] = 4, out[1] = 5, out[2] = 6;
    return 3;
  }
  // FP64: the short lane-pair kernel with shared eigenvectors
  // (SWFD_FLUX_SHARE + 5 blocks per SM, the default; + 4), without
  // (SWFD_FLUX_LOOP + 5, + 4), the unrolled lane-pair kernel
  // (SWFD_FLUX_PAIR + 3..6) and the one-lane kernel (3, 2, 4 blocks per SM)
  out[0] = SWFD_FLUX_DEFAULT64, out[1] = SWFD_FLUX_SHARE + 4, out[2] = SWFD_FLUX_LOOP + 5;
  out[3] = SWFD_FLUX_LOOP + 4, out[4] = SWFD_FLUX_PAIR + 4, out[5] = SWFD_FLUX_PAIR + 3;
  out[6] = SWFD_FLUX_PAIR + 5, out[7] = SWFD_FLUX_PAIR + 6, out[8] = 3, out[9] = 2;
  out[10] = 4;
  return 11;
}

template <class T, int MINB>
static void launch_flux_minb(const Params& p, const T* sp, const T* rp, const DevScalars* dsc,
                             T* fp, int* work, cudaStream_t s) {
  k_flux_xy<T, false, false, MINB><<<flux_grid<T, MINB>(), SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp,
                                                                                    dsc, fp, work);
}

// the flux kernel variant of the problem: rank segments (ex6), limiter
template <class T>
static void launch_flux_xy(const Params& p, const void* split, const void* roe,
                           const DevScalars* dsc, void* flux, int* work, cudaStream_t s) {
  const T* sp = (const T*)split;
  const T* rp = (const T*)roe;
  T* fp = (T*)flux;
  const int grid = flux_grid<T>();
  if constexpr (sizeof(T) == 8) {
    if (p.quad) {  // the binary128 subexpressions of the reference build
      constexpr int M = SWFD_FLUX_MINB(T);
      if (p.seg_alpha && p.limiter)
        k_flux_xy<T, true, true, M, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
      else if (p.seg_alpha)
        k_flux_xy<T, true, false, M, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
      else if (p.limiter)
        k_flux_xy<T, false, true, M, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
      else
        k_flux_xy<T, false, false, M, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
      return;
    }
  }
  // the FP64 default shape is the short lane-pair kernel with shared
  // eigenvectors, 5 blocks per SM (SWFD_FLUX_DEFAULT64); flux_minb 3 selects
  // the one-lane kernel's default
  int minb = p.flux_minb;
  if constexpr (sizeof(T) == 8)
    if (!minb) minb = SWFD_FLUX_DEFAULT64;
  if (!p.seg_alpha && !p.limiter && minb && minb != SWFD_FLUX_MINB(T)) {
    if constexpr (sizeof(T) == 8) {
      if (minb == 2) return launch_flux_minb<T, 2>(p, sp, rp, dsc, fp, work, s);
      if (minb == 4) return launch_flux_minb<T, 4>(p, sp, rp, dsc, fp, work, s);
#define SWFD_PAIR_CASE(M)                                                                    \
  if (minb == SWFD_FLUX_PAIR + M) {                                                          \
    k_flux_xy_pair<M><<<flux_grid_pair<M>(), SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work); \
    return;                                                                                  \
  }
      SWFD_PAIR_CASE(3)
      SWFD_PAIR_CASE(4)
      SWFD_PAIR_CASE(5)
      SWFD_PAIR_CASE(6)
#undef SWFD_PAIR_CASE
#define SWFD_LOOP_CASE(M)                                                                    \
  if (minb == SWFD_FLUX_LOOP + M) {                                                          \
    k_flux_xy_loop<M><<<flux_grid_loop<M>(), SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work); \
    return;                                                                                  \
  }
      SWFD_LOOP_CASE(4)
      SWFD_LOOP_CASE(5)
#undef SWFD_LOOP_CASE
#define SWFD_SHARE_CASE(M)                                                                     \
  if (minb == SWFD_FLUX_SHARE + M) {                                                           \
    k_flux_xy_share<M><<<flux_grid_share<M>(), SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work); \
    return;                                                                                    \
  }
      SWFD_SHARE_CASE(4)
      SWFD_SHARE_CASE(5)
#undef SWFD_SHARE_CASE
    } else {
      if (minb == 5) return launch_flux_minb<T, 5>(p, sp, rp, dsc, fp, work, s);
      if (minb == 6) return launch_flux_minb<T, 6>(p, sp, rp, dsc, fp, work, s);
    }
  }
  if (p.seg_alpha && p.limiter)
    k_flux_xy<T, true, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
  else if (p.seg_alpha)
    k_flux_xy<T, true, false><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
  else if (p.limiter)
    k_flux_xy<T, false, true><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
  else
    k_flux_xy<T, false, false><<<grid, SWFD_FLUX_BLOCK, 0, s>>>(p, sp, rp, dsc, fp, work);
}

cudaError_t launch_flux(const Params& p, const void* split, const void* roe,
                        const DevScalars* dsc, void* flux, int* work, cudaStream_t s) {
  const Geom& g = p.g;
  const bool f32 = p.precision == SWFD_PRECISION_FP32_BULK;
  if (g.ndim == 1) {
    // the 1D eigenvectors come from the state, which the caller passes as roe
    const int64_t lanes = 8 * (int64_t)(g.nx + 2);  // eight lanes per cell
    const int b = cell_block(lanes), gb = (int)((lanes + b - 1) / b);
    // the limiter's counts: den_count and pre_count, adjacent in DevScalars
    unsigned long long* cnt = (unsigned long long*)&const_cast<DevScalars*>(dsc)->den_count;
    if (f32)
      k_flux1d<float><<<gb, b, 0, s>>>(p, (const double*)roe, (const float*)split, (float*)flux,
                                       cnt);
    else if (p.quad)
      k_flux1d<double, true><<<gb, b, 0, s>>>(p, (const double*)roe, (const double*)split,
                                               (double*)flux, cnt);
    else
      k_flux1d<double><<<gb, b, 0, s>>>(p, (const double*)roe, (const double*)split,
                                         (double*)flux, cnt);
    return cudaGetLastError();
  }
  if (f32)
    launch_flux_xy<float>(p, split, roe, dsc, flux, work, s);
  else
    launch_flux_xy<double>(p, split, roe, dsc, flux, work, s);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// scheme + RK stage combination + checkpositivity, one thread per cell.
// Whole-array update as in the reference (RHS = 0 in the ghosts):
//   stage 1  u = u + dt*RHS                          (main.f90:587)
//   stage 2  u = 0.75*u0 + 0.25*(u + dt*RHS)         (main.f90:604)
//   stage 3  u = (u0 + 2*(u + dt*RHS))/3             (main.f90:621)
// The flux difference is formed in T; the RK combination accumulates into the
// FP64 state in both precisions.
// ---------------------------------------------------------------------------
// ox, oy: the cell's offsets in the x and y flux planes (its own rank
// segment's copy; the cell offset itself without segments)
// FP32-bulk RHS of a cell from its flux differences A (x) and B (y)
__device__ __forceinline__ float rhs32(const Params& p, float A, float B, double amd) {
  const float ix = p.fdx_inv, iy = p.fdy_inv;
  if (p.alpha_premul) return -A * ix - B * iy;
  const float am = d2f(amd);
  return -(am * A) * ix - (am * B) * iy;
}
// FP32-bulk RK stage value: the FP64 accumulation with fused multiply-adds
// (u + dt L; 0.75 u0 + 0.25 v; (u0 + 2 v)/3)
__device__ __forceinline__ double rk32_value(int stage, double dt, double r, double u,
                                             const double* u0) {
  double v = fma(dt, r, u);
  if (stage == 2) v = fma(0.75, *u0, 0.25 * v);
  else if (stage == 3) v = fma(2.0, v, *u0) * (1.0 / 3.0);
  return v;
}
// FP32-bulk checkpositivity of a 2D cell: the pressure in FP64 with one
// reciprocal
__device__ __forceinline__ int pos32_bad(const Params& p, const double nv[4]) {
  const double ri = -0.5 * rcp_bulk(nv[0]);
  const double pe = fma(fma(nv[2], nv[2], nv[1] * nv[1]), ri, nv[3]);
  if (p.pos_strict) return (nv[0] < p.eps) || (pe < p.eps);
  return (nv[0] <= p.eps) || (pe <= p.eps);
}

template <class T>
__device__ __forceinline__ T rhs2d(const Params& p, const T* __restrict__ flux, int c, int64_t ox,
                                   int64_t oy, double amd) {
  const int64_t S = p.sg.plane, pit = p.sg.pitch;
  const T* fpf = flux + c * S;
  const T* fnf = flux + (4 + c) * S;
  const T* gpf = flux + (8 + c) * S;
  const T* gnf = flux + (12 + c) * S;
  T A = (ldt(fpf + ox) - ldt(fnf + ox + 1)) - (ldt(fpf + ox - 1) - ldt(fnf + ox));
  T B = (ldt(gpf + oy) - ldt(gnf + oy + pit)) - (ldt(gpf + oy - pit) - ldt(gnf + oy));
  if constexpr (sizeof(T) == 4) {  // FP32-bulk: reciprocals of dx, dy
    return rhs32(p, A, B, amd);
  } else {
    const T dx = T(p.dx), dy = T(p.dy), am = T(amd);
    // (-x)/d == -(x/d): the divisions on the integer pipes (tdiv)
    if (p.alpha_premul) return -tdiv(A, dx) - tdiv(B, dy);  // ex4_sedov_2d/main.f90:644-645
    return -tdiv(am * A, dx) - tdiv(am * B, dy);            // ex3_vortex_accuracy_2d/main.f90:541-542
  }
}

template <class T>
__device__ __forceinline__ T rhs1d(const Params& p, const T* __restrict__ flux, int c, int64_t o,
                                   double amd) {
  // flus(i) = alphamax*(hp_flux(i-1) - hn_flux(i)); RHS = -(flus(i+1)-flus(i))/dx
  const int64_t P = p.g.plane;
  const T* hp = flux + c * P;
  const T* hn = flux + (3 + c) * P;
  return rhs1d_value<T>(p, amd, ldt(hp + o - 1), ldt(hn + o), ldt(hp + o), ldt(hn + o + 1));
}

__device__ __forceinline__ int block_or(int v) { return __syncthreads_or(v); }

// flux difference of interior cell (i, j) of a 2D problem
template <class T>
__device__ __forceinline__ T rhs2d_cell(const Params& p, const T* __restrict__ flux, int c, int i,
                                        int j, double amd) {
  const int sx = p.seg_alpha ? (i - 1) / p.nxl : 0, sy = p.seg_alpha ? (j - 1) / p.nyl : 0;
  return rhs2d<T>(p, flux, c, seg_x_off(p, i, j, sx), seg_y_off(p, i, j, sy), amd);
}


// NC: the components as a compile-time count (4 in 2D, 3 in 1D), so that
// the components' chains are unrolled side by side and nv stays in registers
template <class T, int NC = 4>
__device__ __forceinline__ int rk_cell(const Params& p, int stage, const double* __restrict__ u,
                                       const double* u0, const T* __restrict__ flux, double dt,
                                       double am, double* out, int64_t t) {
  const Geom& g = p.g;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  int bad = 0;
  if (t < ncell) {
    int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
    const int64_t o = g.at(i, j), P = g.plane;
    bool interior = (i >= 1 && i <= g.nx) && (NC == 3 || (j >= 1 && j <= g.ny));
    double nv[4];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      double r = 0.0;
      if (interior)
        r = tod((NC == 3) ? rhs1d<T>(p, flux, c, o, am) : rhs2d_cell<T>(p, flux, c, i, j, am));
      double v;
      if (sizeof(T) == 4) {  // FP32-bulk: the FP64 accumulation with fused multiply-adds
        v = rk32_value(stage, dt, r, ld(u + c * P + o), u0 + c * P + o);
      } else {
        v = ld(u + c * P + o) + dt * r;
        if (stage >= 2) v = rk_combine(p, stage, u0[c * P + o], v);
      }
      nv[c] = v;
      out[c * P + o] = v;
    }
    if (interior) {
      // checkpositivity (ex3_vortex_accuracy_2d/main.f90:640-647,
      // ex2_sedov_1d/main.f90:381-387; `<` in ex4/ex5)
      double pe;
      if (sizeof(T) == 4 && NC == 4) return pos32_bad(p, nv);
      if (sizeof(T) == 4) {  // FP32-bulk: FP64 with one reciprocal
        const double ri = -0.5 * rcp_bulk(nv[0]);
        pe = fma(nv[1] * nv[1], ri, nv[2]);
      } else if (NC == 3) {
        pe = nv[2] - tscale<-1>(tdiv(nv[1] * nv[1], nv[0]));
      } else {
        pe = nv[3] - tscale<-1>(tdiv(nv[2] * nv[2], nv[0])) - tscale<-1>(tdiv(nv[1] * nv[1], nv[0]));
      }
      if (p.pos_strict) bad = (nv[0] < p.eps) || (pe < p.eps);
      else bad = (nv[0] <= p.eps) || (pe <= p.eps);
    }
  }
  return bad;
}

// postag starts the stage at 0 (findalpha clears it).  The last block to
// finish counts the stage and takes its positivity decision: decide 1 sets
// the IF condition hs to postag (the sweep, ex3_vortex_accuracy_2d/main.f90:
// 590-595), decide 2 to !postag (the restart RK's next stage,
// ex2_sedov_1d/main.f90:349-364).
__device__ __forceinline__ void rk_block_done(DevScalars* dsc, int bad, int stage,
                                              cudaGraphConditionalHandle hs, int decide) {
  bad = block_or(bad);
  if (threadIdx.x != 0) return;
  if (bad) atomicOr(&dsc->postag, 1);
  __threadfence();
  if (atomicAdd(&dsc->rk_done, 1) != (int)gridDim.x - 1) return;
  __threadfence();
  const int tag = atomicOr(&dsc->postag, 0);
  dsc->rk_done = 0;
  dsc->rk_runs[stage]++;
  if (decide == 1) set_cond(hs, &dsc->cond, tag ? 1u : 0u);
  else if (decide == 2) set_cond(hs, &dsc->cond, tag ? 0u : 1u);
}

template <class T>
__global__ void k_rk(Params p, int stage, const double* __restrict__ u, const double* u0,
                     const T* __restrict__ flux, DevScalars* dsc, double* out,
                     cudaGraphConditionalHandle hs, int decide) {
  int bad = rk_cell<T>(p, stage, u, u0, flux, dsc->dt, dsc->alphamax, out,
                       (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  rk_block_done(dsc, bad, stage, hs, decide);
}

// 1D: four lanes per cell, lane c < 3 forming component c (its RHS and RK
// combination are a chain of their own), lane 0 testing the cell's
// positivity from the three new values; the expressions are rk_cell's.
// lane t (every lane of its warp takes part: the group's shuffles); returns
// the positivity flag of lane 0 of an interior cell's group
template <class T>
__device__ __forceinline__ int rk1d_lane(const Params& p, int stage, const double* __restrict__ u,
                                         const double* u0, const T* __restrict__ flux, double dt,
                                         double amd, double* out, int64_t t) {
  const Geom& g = p.g;
  const int cell = (int)(t >> 2), c = (int)(t & 3);
  const bool in_grid = cell < g.LI;
  const int i = cell - 2;
  const bool interior = in_grid && i >= 1 && i <= g.nx;
  const int64_t P = g.plane, o = in_grid ? g.at(i, -2) : 0;
  double v = 0.0;
  if (in_grid && c < 3) {
    double r = 0.0;
    if (interior) r = tod(rhs1d<T>(p, flux, c, o, amd));
    v = rk1d_value<T>(p, stage, dt, r, ld(u + c * P + o), u0 + c * P + o);
    out[c * P + o] = v;
  }
  const int base = threadIdx.x & ~3 & 31;
  const double n0 = __shfl_sync(0xffffffffu, v, base), n1 = __shfl_sync(0xffffffffu, v, base + 1),
               n2 = __shfl_sync(0xffffffffu, v, base + 2);
  int bad = 0;
  if (interior && c == 0) bad = pos1d_bad<T>(p, n0, n1, n2);
  return bad;
}

template <class T>
__global__ void k_rk1d(Params p, int stage, const double* __restrict__ u, const double* u0,
                       const T* __restrict__ flux, DevScalars* dsc, double* out,
                       cudaGraphConditionalHandle hs, int decide) {
  const int bad = rk1d_lane<T>(p, stage, u, u0, flux, dsc->dt, dsc->alphamax, out,
                               (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  rk_block_done(dsc, bad, stage, hs, decide);
}

cudaError_t launch_rk(const Params& p, int stage, const double* u, const double* u0,
                      const void* flux, const DevScalars* dsc, double* out, cudaStream_t s,
                      cudaGraphConditionalHandle hs, int decide) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  if (p.g.ndim == 1) {  // four lanes per cell
    const int64_t lanes = 4 * n;
    const int b = cell_block(lanes);
    const unsigned gb = (unsigned)((lanes + b - 1) / b);
    if (p.precision == SWFD_PRECISION_FP32_BULK)
      k_rk1d<float><<<gb, b, 0, s>>>(p, stage, u, u0, (const float*)flux,
                                     const_cast<DevScalars*>(dsc), out, hs, decide);
    else
      k_rk1d<double><<<gb, b, 0, s>>>(p, stage, u, u0, (const double*)flux,
                                      const_cast<DevScalars*>(dsc), out, hs, decide);
    return cudaGetLastError();
  }
  const int b = cell_block(n, p.heavy_block);
  const unsigned gb = (unsigned)((n + b - 1) / b);
  if (p.precision == SWFD_PRECISION_FP32_BULK)
    k_rk<float><<<gb, b, 0, s>>>(p, stage, u, u0, (const float*)flux,
                                 const_cast<DevScalars*>(dsc), out, hs, decide);
  else
    k_rk<double><<<gb, b, 0, s>>>(p, stage, u, u0, (const double*)flux,
                                  const_cast<DevScalars*>(dsc), out, hs, decide);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP32-bulk fused stage (2D, no rank segments, no limiter): two kernels per RK
// stage instead of four.
//   k_alpha_terms32: [bc,] findalpha [and dt], and per cell the nine
//     splitting terms (Terms32) and the Roe planes -- the FP64 work of the
//     splitting, once per cell.
//   k_stage32: per tile of 32 x 8 interior cells, the split fluxes of the tile
//     and its stencil halo formed in shared memory from the terms and this
//     stage's alpha, the interface fluxes of every face the tile's cells
//     difference, then the RHS, the RK combination and checkpositivity of the
//     tile's cells; the split, Roe and flux planes of the separate kernels
//     never go through memory.  Every value is formed by the same functions as
//     the separate kernels' (split32/split_pm, roe_eigen2d, weno8_f32,
//     back_project, rhs32, rk32_value, pos32_bad), so both give the same bits.
// Terms planes (floats, plane pitch of the state): fr fm fn fe f1 fxy f3 g2 g3.
// ---------------------------------------------------------------------------
template <bool NC>
__device__ __forceinline__ void terms32_cell(const Params& p, const double* __restrict__ u,
                                             float* __restrict__ terms, float* __restrict__ roe,
                                             int64_t t) {
  const Geom& g = p.g;
  if (t >= (int64_t)g.LI * g.LJ) return;
  const int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  const int64_t o = g.at(i, j), P = g.plane;
  const double rho = ldc<NC>(u + o), mx = ldc<NC>(u + P + o), my = ldc<NC>(u + 2 * P + o),
               e = ldc<NC>(u + 3 * P + o);
  const double ri = rcp_bulk(rho);
  Prim32 q;
  const Terms32 tm = terms32(p, rho, mx, my, e, ri, q);
  terms[0 * P + o] = tm.fr;
  terms[1 * P + o] = tm.fm;
  terms[2 * P + o] = tm.fn;
  terms[3 * P + o] = tm.fe;
  terms[4 * P + o] = tm.f1;
  terms[5 * P + o] = tm.fxy;
  terms[6 * P + o] = tm.f3;
  terms[7 * P + o] = tm.g2;
  terms[8 * P + o] = tm.g3;
  roe32_store(p, rho, mx, my, e, ri, q, tm.fr, roe, P, o, 3);
}

// BC: the stage-2/3 form (bc of the previous stage's output first; a ghost
// cell's values are then read back with coherent loads)
template <bool BC>
__global__ void k_alpha_terms32(Params p, double* __restrict__ u, DevScalars* dsc, int with_dt,
                                float* __restrict__ terms, float* __restrict__ roe) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (BC) bc2d_cell(p, u, t);
  double a = alpha_cell<!BC, true>(p, u, t);
  terms32_cell<!BC>(p, u, terms, roe, t);
  a = block_max(a);
  if (threadIdx.x != 0) return;
  alpha_last_block(p, dsc, a, with_dt);
}

cudaError_t launch_alpha_terms32(const Params& p, double* u, DevScalars* dsc, cudaStream_t s,
                                 bool bc, bool with_dt, void* terms, void* roe) {
  const int64_t n = (int64_t)p.g.LI * p.g.LJ;
  const int b = cell_block(n);
  const unsigned gb = (unsigned)((n + b - 1) / b);
  if (bc)
    k_alpha_terms32<true><<<gb, b, 0, s>>>(p, u, dsc, with_dt, (float*)terms, (float*)roe);
  else
    k_alpha_terms32<false><<<gb, b, 0, s>>>(p, u, dsc, with_dt, (float*)terms, (float*)roe);
  return cudaGetLastError();
}

#define S32_TX 32
#define S32_TY 8
struct Stage32Tile {
  float xs[8][S32_TY][S32_TX + 6];  // fp (0..3), fn (4..7) of columns i0-3 .. i0+TX+2
  float ys[8][S32_TY + 6][S32_TX];  // gp, gn of rows j0-3 .. j0+TY+2
  float rx[4][S32_TY][S32_TX + 3];  // x-pass Roe planes of columns i0-1 .. i0+TX+1
  float ry[4][S32_TY + 3][S32_TX];  // y-pass Roe planes of rows j0-1 .. j0+TY+1
  float fx[8][S32_TY][S32_TX + 2];  // x faces i0-1 .. i0+TX: op (0..3), on (4..7)
  float fy[8][S32_TY + 2][S32_TX];  // y faces j0-1 .. j0+TY
};

__host__ __device__ __forceinline__ int stage32_tiles(const Geom& g) {
  return ((g.nx + S32_TX - 1) / S32_TX) * ((g.ny + S32_TY - 1) / S32_TY);
}
// ghost cells (three layers around the interior): rows -2..0 and ny+1..ny+3
// over the full width, then columns -2..0 and nx+1..nx+3 of rows 1..ny
__host__ __device__ __forceinline__ int64_t stage32_ghosts(const Geom& g) {
  return 6 * (int64_t)g.LI + 6 * (int64_t)g.ny;
}

// the RK combination of ghost chunk kk (NT consecutive ghost cells) with a
// zero RHS, as rk_cell does for the ghost cells
template <int NT>
__device__ __forceinline__ void stage32_ghosts_chunk(const Params& p, int stage,
                                                     const double* __restrict__ u,
                                                     const double* u0, double dt, double* out,
                                                     int64_t kk) {
  const Geom& g = p.g;
  const int64_t P = g.plane;
  const int64_t k = kk * NT + threadIdx.x;
  if (k >= stage32_ghosts(g)) return;
  int i, j;
  const int64_t band = 3 * (int64_t)g.LI;
  if (k < 2 * band) {
    const int64_t r = k < band ? k : k - band;
    j = (int)(r / g.LI) + (k < band ? -2 : g.ny + 1);
    i = (int)(r % g.LI) - 2;
  } else {
    const int64_t r = k - 2 * band;
    const int c = (int)(r % 6);
    j = (int)(r / 6) + 1;
    i = c < 3 ? c - 2 : g.nx + c - 2;
  }
  const int64_t o = g.at(i, j);
#pragma unroll
  for (int c = 0; c < 4; ++c)
    out[c * P + o] = rk32_value(stage, dt, 0.0, ld(u + c * P + o), u0 + c * P + o);
}

// one 32 x 8 tile of the fused stage; returns this thread's positivity flag.
// Every thread of the block calls it (it synchronises the block).
template <int NT>
__device__ __forceinline__ int stage32_tile(const Params& p, int stage,
                                            const double* __restrict__ u, const double* u0,
                                            const float* __restrict__ terms,
                                            const float* __restrict__ roe, double dt, double amd,
                                            double* out, int tile, Stage32Tile& sm) {
  const Geom& g = p.g;
  const int64_t P = g.plane;
  const int tid = threadIdx.x;
  const int tiles_x = (g.nx + S32_TX - 1) / S32_TX;
  int bad = 0;
  const int i0 = 1 + (tile % tiles_x) * S32_TX, j0 = 1 + (tile / tiles_x) * S32_TY;
  const int nxv = min(S32_TX, g.nx - i0 + 1), nyv = min(S32_TY, g.ny - j0 + 1);
  // phase 1: split fluxes and Roe planes of the tile and its halo
  {
    const float ram = 1.f / d2f(amd);
    const int wxs = nxv + 6, wrx = nxv + 3;
    const int n1 = nyv * wxs, n2 = n1 + (nyv + 6) * nxv, n3 = n2 + nyv * wrx,
              n4 = n3 + (nyv + 3) * nxv;
    const float* ry_src = roe + (p.roe_reg_ex4 ? 4 * P : 0);
    for (int k = tid; k < n4; k += NT) {
      if (k < n1) {
        const int r = k / wxs, c = k - r * wxs;
        const int64_t o = g.at(i0 - 3 + c, j0 + r);
        const float fr = terms[o], fm = terms[P + o], fn = terms[2 * P + o],
                    fe = terms[3 * P + o], f1 = terms[4 * P + o], fxy = terms[5 * P + o],
                    f3 = terms[6 * P + o];
        split_pm(fr, fm, ram, sm.xs[0][r][c], sm.xs[4][r][c]);
        split_pm(fm, f1, ram, sm.xs[1][r][c], sm.xs[5][r][c]);
        split_pm(fn, fxy, ram, sm.xs[2][r][c], sm.xs[6][r][c]);
        split_pm(fe, f3, ram, sm.xs[3][r][c], sm.xs[7][r][c]);
      } else if (k < n2) {
        const int kk = k - n1, r = kk / nxv, c = kk - r * nxv;
        const int64_t o = g.at(i0 + c, j0 - 3 + r);
        const float fr = terms[o], fm = terms[P + o], fn = terms[2 * P + o],
                    fe = terms[3 * P + o], fxy = terms[5 * P + o], g2 = terms[7 * P + o],
                    g3 = terms[8 * P + o];
        split_pm(fr, fn, ram, sm.ys[0][r][c], sm.ys[4][r][c]);
        split_pm(fm, fxy, ram, sm.ys[1][r][c], sm.ys[5][r][c]);
        split_pm(fn, g2, ram, sm.ys[2][r][c], sm.ys[6][r][c]);
        split_pm(fe, g3, ram, sm.ys[3][r][c], sm.ys[7][r][c]);
      } else if (k < n3) {
        const int kk = k - n2, r = kk / wrx, c = kk - r * wrx;
        const int64_t o = g.at(i0 - 1 + c, j0 + r);
#pragma unroll
        for (int q = 0; q < 4; ++q) sm.rx[q][r][c] = roe[q * P + o];
      } else {
        const int kk = k - n3, r = kk / nxv, c = kk - r * nxv;
        const int64_t o = g.at(i0 + c, j0 - 1 + r);
#pragma unroll
        for (int q = 0; q < 4; ++q) sm.ry[q][r][c] = ry_src[q * P + o];
      }
    }
  }
  __syncthreads();
  // phase 2: the faces.  x faces first, their count rounded up to whole warps
  // so that no warp mixes the two directions.
  {
    const float g1 = (float)p.gamma1, weps = (float)p.weno_eps;
    const float am = p.alpha_premul ? (float)amd : 1.f;
    const int wfx = nxv + 2, nfx = nyv * wfx, nfx_pad = (nfx + 31) & ~31;
    const int nf = nfx_pad + (nyv + 2) * nxv;
    for (int k = tid; k < nf; k += NT) {
      float a[5][4], b[5][4], op[4], on[4];
      if (k < nfx_pad) {
        if (k >= nfx) continue;
        const int r = k / wfx, f = k - r * wfx;
        Eigen2D<float> E;
        roe_eigen2d<float>(g1, 0, sm.rx[0][r][f], sm.rx[0][r][f + 1], sm.rx[1][r][f],
                           sm.rx[1][r][f + 1], sm.rx[2][r][f], sm.rx[2][r][f + 1],
                           sm.rx[3][r][f], sm.rx[3][r][f + 1], E);
#pragma unroll
        for (int m = 0; m < 5; ++m)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            a[m][c] = sm.xs[c][r][f + m];
            b[m][c] = sm.xs[4 + c][r][f + m];
          }
        float ur[4], ul[4];
        weno8_f32<0>(E, a, b, weps, ur, ul);
        back_project<0, float>(E, ur, ul, op, on);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          sm.fx[c][r][f] = p.alpha_premul ? am * op[c] : op[c];
          sm.fx[4 + c][r][f] = p.alpha_premul ? am * on[c] : on[c];
        }
      } else {
        const int kk = k - nfx_pad, f = kk / nxv, c0 = kk - f * nxv;
        Eigen2D<float> E;
        roe_eigen2d<float>(g1, 1, sm.ry[0][f][c0], sm.ry[0][f + 1][c0], sm.ry[1][f][c0],
                           sm.ry[1][f + 1][c0], sm.ry[2][f][c0], sm.ry[2][f + 1][c0],
                           sm.ry[3][f][c0], sm.ry[3][f + 1][c0], E);
#pragma unroll
        for (int m = 0; m < 5; ++m)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            a[m][c] = sm.ys[c][f + m][c0];
            b[m][c] = sm.ys[4 + c][f + m][c0];
          }
        float ur[4], ul[4];
        weno8_f32<1>(E, a, b, weps, ur, ul);
        back_project<1, float>(E, ur, ul, op, on);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          sm.fy[c][f][c0] = p.alpha_premul ? am * op[c] : op[c];
          sm.fy[4 + c][f][c0] = p.alpha_premul ? am * on[c] : on[c];
        }
      }
    }
  }
  __syncthreads();
  // phase 3: RHS, RK combination and checkpositivity of the tile's cells
  {
    const int r = tid / S32_TX, c = tid % S32_TX;
    if (r < nyv && c < nxv) {
      const int64_t o = g.at(i0 + c, j0 + r);
      double nv[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float A = (sm.fx[k][r][c + 1] - sm.fx[4 + k][r][c + 2]) -
                        (sm.fx[k][r][c] - sm.fx[4 + k][r][c + 1]);
        const float B = (sm.fy[k][r + 1][c] - sm.fy[4 + k][r + 2][c]) -
                        (sm.fy[k][r][c] - sm.fy[4 + k][r + 1][c]);
        const double v =
            rk32_value(stage, dt, tod(rhs32(p, A, B, amd)), ld(u + k * P + o), u0 + k * P + o);
        nv[k] = v;
        out[k * P + o] = v;
      }
      bad = pos32_bad(p, nv);
    }
  }
  return bad;
}

// NT threads per tile (256: three rounds of faces; 320: two), MINB resident
// tiles per SM.  Blocks past the tiles run the ghost cells' RK combination.
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    k_stage32(Params p, int stage, const double* __restrict__ u, const double* u0,
              const float* __restrict__ terms, const float* __restrict__ roe, DevScalars* dsc,
              double* out, cudaGraphConditionalHandle hs, int decide) {
  extern __shared__ __align__(16) unsigned char s32_raw[];
  Stage32Tile& sm = *reinterpret_cast<Stage32Tile*>(s32_raw);
  const double dt = dsc->dt, amd = dsc->alphamax;
  const int tiles = stage32_tiles(p.g);
  int bad = 0;
  if ((int)blockIdx.x >= tiles)
    stage32_ghosts_chunk<NT>(p, stage, u, u0, dt, out, (int64_t)blockIdx.x - tiles);
  else
    bad = stage32_tile<NT>(p, stage, u, u0, terms, roe, dt, amd, out, (int)blockIdx.x, sm);
  rk_block_done(dsc, bad, stage, hs, decide);
}

size_t stage32_smem_bytes() { return sizeof(Stage32Tile); }

cudaError_t batch_stage32_setup();
// the launch shapes (threads per tile, tiles per SM): 1 = 256 x 2,
// 2 = 320 x 2, 3 = 256 x 3, 4 = 256 x 4 (the default: 64 registers, the
// fastest on the 360^2 and 1024^2 vortex), 5 = 320 x 3
cudaError_t stage32_setup() {
  const int b = (int)sizeof(Stage32Tile);
  cudaError_t e = cudaFuncSetAttribute(k_stage32<256, 2>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage32<320, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage32<256, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage32<256, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_stage32<320, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
  if (e == cudaSuccess) e = batch_stage32_setup();
  return e;
}

template <int NT, int MINB>
static void stage32_go(const Params& p, int stage, const double* u, const double* u0,
                       const void* terms, const void* roe, DevScalars* dsc, double* out,
                       cudaStream_t s, cudaGraphConditionalHandle hs, int decide) {
  const int64_t blocks = stage32_tiles(p.g) + (stage32_ghosts(p.g) + NT - 1) / NT;
  k_stage32<NT, MINB><<<(unsigned)blocks, NT, sizeof(Stage32Tile), s>>>(
      p, stage, u, u0, (const float*)terms, (const float*)roe, dsc, out, hs, decide);
}

cudaError_t launch_stage32(const Params& p, int shape, int stage, const double* u,
                           const double* u0, const void* terms, const void* roe, DevScalars* dsc,
                           double* out, cudaStream_t s, cudaGraphConditionalHandle hs,
                           int decide) {
  if (shape == 1) stage32_go<256, 2>(p, stage, u, u0, terms, roe, dsc, out, s, hs, decide);
  else if (shape == 2) stage32_go<320, 2>(p, stage, u, u0, terms, roe, dsc, out, s, hs, decide);
  else if (shape == 3) stage32_go<256, 3>(p, stage, u, u0, terms, roe, dsc, out, s, hs, decide);
  else if (shape == 5) stage32_go<320, 3>(p, stage, u, u0, terms, roe, dsc, out, s, hs, decide);
  else stage32_go<256, 4>(p, stage, u, u0, terms, roe, dsc, out, s, hs, decide);
  return cudaGetLastError();
}

template <class T>
__global__ void k_rhs(Params p, const T* __restrict__ flux, const DevScalars* dsc,
                      double* __restrict__ rhs) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  if (t >= ncell) return;
  int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  const int64_t o = g.at(i, j), P = g.plane;
  bool interior = (i >= 1 && i <= g.nx) && (g.ndim == 1 || (j >= 1 && j <= g.ny));
  for (int c = 0; c < g.nc; ++c) {
    double r = 0.0;
    if (interior)
      r = tod((g.ndim == 1) ? rhs1d<T>(p, flux, c, o, dsc->alphamax)
                                 : rhs2d_cell<T>(p, flux, c, i, j, dsc->alphamax));
    rhs[c * P + o] = r;
  }
}

cudaError_t launch_rhs(const Params& p, const void* flux, const DevScalars* dsc, double* rhs,
                       cudaStream_t s) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  const unsigned gb = (unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK);
  if (p.precision == SWFD_PRECISION_FP32_BULK)
    k_rhs<float><<<gb, SWFD_BLOCK, 0, s>>>(p, (const float*)flux, dsc, rhs);
  else
    k_rhs<double><<<gb, SWFD_BLOCK, 0, s>>>(p, (const double*)flux, dsc, rhs);
  return cudaGetLastError();
}

__global__ void k_positivity(Params p, const double* __restrict__ u, DevScalars* dsc) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  int bad = 0;
  if (t < ncell) {
    int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
    const int64_t o = g.at(i, j), P = g.plane;
    bool interior = (i >= 1 && i <= g.nx) && (g.ndim == 1 || (j >= 1 && j <= g.ny));
    if (interior) {
      double pe, r = ld(u + o);
      if (g.ndim == 1) {
        double m = ld(u + P + o);
        pe = ld(u + 2 * P + o) - m * m / r / 2.;
      } else {
        double mx = ld(u + P + o), my = ld(u + 2 * P + o);
        pe = ld(u + 3 * P + o) - my * my / r / 2. - mx * mx / r / 2.;
      }
      if (p.pos_strict) bad = (r < p.eps) || (pe < p.eps);
      else bad = (r <= p.eps) || (pe <= p.eps);
    }
  }
  if (block_or(bad) && threadIdx.x == 0) atomicOr(&dsc->postag, 1);
}

cudaError_t launch_positivity(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  cudaError_t e = cudaMemsetAsync(&dsc->postag, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  k_positivity<<<(unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(p, u, dsc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// layout conversion between u(nc,-2:nx+3,-2:ny+3) and the SoA planes
// ---------------------------------------------------------------------------
__global__ void k_f2s(Params p, const double* __restrict__ src, double* __restrict__ dst) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  if (t >= ncell) return;
  int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  for (int c = 0; c < g.nc; ++c) dst[c * g.plane + g.at(i, j)] = src[t * g.nc + c];
}
__global__ void k_s2f(Params p, const double* __restrict__ src, double* __restrict__ dst) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t ncell = (int64_t)g.LI * g.LJ;
  if (t >= ncell) return;
  int i = ((int)t % g.LI) - 2, j = ((int)t / g.LI) - 2;
  for (int c = 0; c < g.nc; ++c) dst[t * g.nc + c] = src[c * g.plane + g.at(i, j)];
}
cudaError_t launch_fortran_to_soa(const Params& p, const double* src, double* dst, cudaStream_t s) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  k_f2s<<<(unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(p, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_soa_to_fortran(const Params& p, const double* src, double* dst, cudaStream_t s) {
  int64_t n = (int64_t)p.g.LI * p.g.LJ;
  k_s2f<<<(unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(p, src, dst);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// batch of scalar WENO5 reconstructions (the MODULE weno5 entry points)
// ---------------------------------------------------------------------------
__global__ void k_weno_batch(const double* __restrict__ st, int64_t n, double eps, int quad,
                             QuadWeno qw, double* __restrict__ ul, double* __restrict__ ur) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* a = st + 5 * k;
  if (quad) {
    if (ul) ul[k] = weno_left_qd(a[0], a[1], a[2], a[3], a[4], qw);
    if (ur) ur[k] = weno_right_qd(a[0], a[1], a[2], a[3], a[4], qw);
    return;
  }
  if (ul) ul[k] = weno_left<double>(a[0], a[1], a[2], a[3], a[4], eps);
  if (ur) ur[k] = weno_right<double>(a[0], a[1], a[2], a[3], a[4], eps);
}
cudaError_t launch_weno_batch(const double* st, int64_t n, double eps, int quad, double* ul,
                              double* ur, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  QuadWeno qw;
  qw.c1312 = qd::div(qd::from_double(13.0), qd::from_double(12.0));
  qw.eps = qd::div(qd::from_double(1.0), qd::from_double(eps == 1e-12 ? 1e12 : 1e6));
  k_weno_batch<<<(unsigned)((n + SWFD_BLOCK - 1) / SWFD_BLOCK), SWFD_BLOCK, 0, s>>>(
      st, n, eps, quad, qw, ul, ur);
  return cudaGetLastError();
}

}  // namespace swfd

// ===========================================================================
// Batched stage kernels.  blockIdx.y indexes the slot table (grid.x strides
// over the slot's cells); slots that are not active are skipped.  The per
// cell arithmetic is the single-instance code above.
// ===========================================================================
namespace swfd {

__global__ void kb_stage_reset(BatchSlot* __restrict__ tab, BatchCtl* ctl, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    ctl->any_postag = 0;
    ctl->flux_work = 0;
  }
  if (s >= n || !tab[s].active) return;
  tab[s].dsc->alpha_bits = 0;
  tab[s].dsc->postag = 0;
}

// The per-cell batched kernels walk the running slots' cells as equal tiles
// of ctl->tile_cells cells (the last tile of a slot may be short): tile k
// belongs to the slot s with tp[s] <= k < tp[s+1].  A persistent grid takes
// the tiles round robin, so every block does the same work whatever the mix
// of grid sizes.
__device__ __forceinline__ int tile_slot(const long long* __restrict__ tp, int n, long long k) {
  int lo = 0, hi = n - 1;  // last slot with tp[s] <= k
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tp[mid] <= k) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void kb_alpha(const BatchSlot* __restrict__ tab, const long long* __restrict__ tp,
                         int n, const BatchCtl* __restrict__ ctl, int in) {
  const long long total = ctl->total_tiles;
  const int tc = ctl->tile_cells;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(tp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;  // uniform over the block
    const long long c0 = (k - tp[s]) * tc, c1 = min(c0 + tc, sl.ncell);
    double a = 0.0;
    for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x) {
      const double at = alpha_cell(sl.p, sl.st[in], t);
      alpha_store(sl.p, t, at);
      a = fmax(a, at);
    }
    a = block_max(a);
    if (threadIdx.x == 0)
      atomicMax(&sl.dsc->alpha_bits, (unsigned long long)__double_as_longlong(a));
    __syncthreads();  // block_max's shared words are reused by the next tile
  }
}

__global__ void kb_alpha_final(const BatchSlot* __restrict__ tab, int n, int stage) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !tab[s].active) return;
  alpha_final_body(tab[s].dsc);
  if (stage == 1) dt_body(tab[s].p, tab[s].dsc);
}

template <class T>
// pass 1: the x part of slots with rank segments, everything of the others;
// pass 2: the y part of slots with rank segments (after their y wall mirror)
__global__ void kb_prep(const BatchSlot* __restrict__ tab, const long long* __restrict__ tp, int n,
                        const BatchCtl* __restrict__ ctl, int in, int pass) {
  const long long total = ctl->total_tiles;
  const int tc = ctl->tile_cells;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(tp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;
    const int which = sl.p.seg_alpha ? pass : (pass == 1 ? 3 : 0);
    if (!which) continue;
    const double am = sl.dsc->alphamax;
    const long long c0 = (k - tp[s]) * tc, c1 = min(c0 + tc, sl.ncell);
    for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x)
      prep2d_cell<T>(sl.p, sl.st[in], am, (T*)sl.split, (T*)sl.roe, t, which);
  }
}

// ex6 slots: alpha per rank row / column and the wall mirrors
__global__ void kb_seg_alpha(const BatchSlot* __restrict__ tab) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!sl.active || !sl.p.seg_alpha) return;
  const int64_t n = seg_alpha_items(sl.p);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    seg_alpha_item(sl.p, t);
}
__global__ void kb_walls(const BatchSlot* __restrict__ tab, int in, int ydir) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!sl.active || sl.p.problem != SWFD_PROBLEM_SHOCK_DIFFRACTION) return;
  const int n = ydir ? sl.p.total * 3 : (min(6 * sl.p.total, sl.p.g.ny + 1) + 1) * 3;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    if (ydir) wall_y_item(sl.p, sl.st[in], t);
    else wall_x_item(sl.p, sl.st[in], t);
  }
}

// all slots' interfaces in one persistent launch; chunk c belongs to the slot
// whose [prefix[s], prefix[s+1]) holds it
template <class T>
__global__ void __launch_bounds__(SWFD_FLUX_BLOCK, SWFD_FLUX_MINB(T))
    kb_flux(const BatchSlot* __restrict__ tab, const long long* __restrict__ prefix, int n,
            BatchCtl* ctl) {
  const int lane = threadIdx.x & 31;
  const long long total = ctl->total_chunks;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(&ctl->flux_work, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= total) break;
    int lo = 0, hi = n - 1;  // last slot with prefix[s] <= c
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (prefix[mid] <= c) lo = mid;
      else hi = mid - 1;
    }
    const BatchSlot& sl = tab[lo];
    if (!sl.active) continue;
    const T am = sl.p.alpha_premul ? T(sl.dsc->alphamax) : T(1.0);
    flux_chunk<T, true>(sl.p, (const T*)sl.split, (const T*)sl.roe, am, (T*)sl.flux, c - prefix[lo],
                  sl.chunks_x, lane,
                        (unsigned long long*)&sl.dsc->den_count, flux_const<T>(sl.p));
  }
}

template <class T>
__global__ void kb_rk(const BatchSlot* __restrict__ tab, const long long* __restrict__ tp, int n,
                      BatchCtl* ctl, int stage, int in, int out) {
  const long long total = ctl->total_tiles;
  const int tc = ctl->tile_cells;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(tp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;
    DevScalars* d = sl.dsc;
    const double dt = d->dt, am = d->alphamax;
    const long long c0 = (k - tp[s]) * tc, c1 = min(c0 + tc, sl.ncell);
    int bad = 0;
    for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x)
      bad |= sl.p.g.ndim == 1 ? rk_cell<T, 3>(sl.p, stage, sl.st[in], sl.st[0], (const T*)sl.flux,
                                             dt, am, sl.st[out], t)
                              : rk_cell<T, 4>(sl.p, stage, sl.st[in], sl.st[0], (const T*)sl.flux,
                                             dt, am, sl.st[out], t);
    if (block_or(bad) && threadIdx.x == 0) {
      atomicOr(&d->postag, 1);
      if (sl.use_limiter == 2) atomicOr(&ctl->any_postag, 1);
    }
  }
}

__global__ void kb_bc(const BatchSlot* __restrict__ tab, const long long* __restrict__ tp, int n,
                      const BatchCtl* __restrict__ ctl, int out) {
  const long long total = ctl->total_tiles;
  const int tc = ctl->tile_cells;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(tp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;
    const long long c0 = (k - tp[s]) * tc, c1 = min(c0 + tc, sl.ncell);
    for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x) bc2d_cell(sl.p, sl.st[out], t);
  }
}

// time = time + dt; an instance that reaches its T (or hits an error) stops
__global__ void kb_time_advance(BatchSlot* __restrict__ tab, BatchCtl* ctl, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !tab[s].active) return;
  DevScalars* d = tab[s].dsc;
  d->time = d->time + d->dt;
  d->steps++;
  if (!(d->time <= d->t_end - 1e-10) || d->error) {
    tab[s].active = 0;
    atomicSub(&ctl->n_active, 1);
  }
}

__global__ void kb_cond_any_postag(cudaGraphConditionalHandle h, BatchCtl* ctl) {
  set_cond(h, &ctl->cond, ctl->any_postag ? 1u : 0u);
}

__global__ void kb_run_cond(cudaGraphConditionalHandle h, BatchCtl* ctl, int advance) {
  if (advance) ctl->steps++;
  set_cond(h, &ctl->cond, (ctl->n_active > 0 && ctl->steps < ctl->steps_limit) ? 1u : 0u);
}

// persistent grid of the tiled per-cell kernels: 8 blocks of 256 per SM
static int batch_tile_grid() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid = 8 * (sms > 0 ? sms : 1);
  }
  return grid;
}

static int batch_grid_x(int n_slots, long long max_cell) {
  long long want = (4096 + n_slots - 1) / n_slots;
  long long cap = (max_cell + SWFD_BLOCK - 1) / SWFD_BLOCK;
  long long x = want < 64 ? 64 : want;
  if (x > cap) x = cap;
  return (int)(x < 1 ? 1 : x);
}

cudaError_t launch_batch_stage(const BatchLaunch& b, int stage, int in, int out,
                               cudaGraphConditionalHandle h_sweep, cudaStream_t s) {
  const int n = b.n_slots;
  const int gs = (n + 127) / 128;
  const dim3 grid(batch_grid_x(n, b.max_cell), n);
  const int tg = batch_tile_grid();
  kb_stage_reset<<<gs, 128, 0, s>>>(b.tab, b.ctl, n);
  kb_alpha<<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in);
  kb_alpha_final<<<gs, 128, 0, s>>>(b.tab, n, stage);
  if (b.segmented) {
    kb_seg_alpha<<<grid, SWFD_BLOCK, 0, s>>>(b.tab);
    kb_walls<<<dim3(1, n), 256, 0, s>>>(b.tab, in, 0);
  }
  if (b.fp32) {
    kb_prep<float><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in, 1);
    if (b.segmented) {
      kb_walls<<<dim3(1, n), 256, 0, s>>>(b.tab, in, 1);
      kb_prep<float><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in, 2);
    }
    kb_flux<float><<<flux_grid<float>(), SWFD_FLUX_BLOCK, 0, s>>>(b.tab, b.prefix, n, b.ctl);
    kb_rk<float><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, stage, in, out);
  } else {
    kb_prep<double><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in, 1);
    if (b.segmented) {
      kb_walls<<<dim3(1, n), 256, 0, s>>>(b.tab, in, 1);
      kb_prep<double><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in, 2);
    }
    kb_flux<double><<<flux_grid<double>(), SWFD_FLUX_BLOCK, 0, s>>>(b.tab, b.prefix, n, b.ctl);
    kb_rk<double><<<tg, SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, stage, in, out);
  }
  if (h_sweep) kb_cond_any_postag<<<1, 1, 0, s>>>(h_sweep, b.ctl);
  return cudaGetLastError();
}

// The fused FP32-bulk stage over the batch: findalpha with each cell's
// splitting terms (kb_alpha's tiles), then k_stage32's tiles and ghost chunks
// of all running slots taken round robin by a persistent grid (the slot of
// item k: s32prefix[s] <= k < s32prefix[s+1]); each slot's positivity flag as
// kb_rk sets it.
__global__ void kb_alpha_terms32(const BatchSlot* __restrict__ tab,
                                 const long long* __restrict__ tp, int n,
                                 const BatchCtl* __restrict__ ctl, int in) {
  const long long total = ctl->total_tiles;
  const int tc = ctl->tile_cells;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(tp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;  // uniform over the block
    const long long c0 = (k - tp[s]) * tc, c1 = min(c0 + tc, sl.ncell);
    double a = 0.0;
    for (long long t = c0 + threadIdx.x; t < c1; t += blockDim.x) {
      a = fmax(a, alpha_cell<true, true>(sl.p, sl.st[in], t));
      terms32_cell<true>(sl.p, sl.st[in], (float*)sl.split, (float*)sl.roe, t);
    }
    a = block_max(a);
    if (threadIdx.x == 0)
      atomicMax(&sl.dsc->alpha_bits, (unsigned long long)__double_as_longlong(a));
    __syncthreads();  // block_max's shared words are reused by the next tile
  }
}

long long stage32_items(const Params& p) {
  return stage32_tiles(p.g) + (stage32_ghosts(p.g) + 255) / 256;
}

__global__ void __launch_bounds__(256, 4)
    kb_stage32(const BatchSlot* __restrict__ tab, const long long* __restrict__ sp, int n,
               BatchCtl* ctl, int stage, int in, int out) {
  extern __shared__ __align__(16) unsigned char s32_raw[];
  Stage32Tile& sm = *reinterpret_cast<Stage32Tile*>(s32_raw);
  const long long total = ctl->total_s32;
  for (long long k = blockIdx.x; k < total; k += gridDim.x) {
    const int s = tile_slot(sp, n, k);
    const BatchSlot& sl = tab[s];
    if (!sl.active) continue;  // uniform over the block
    DevScalars* d = sl.dsc;
    const double dt = d->dt, am = d->alphamax;
    const long long local = k - sp[s];
    const int tiles = stage32_tiles(sl.p.g);
    if (local < tiles) {
      const int bad = stage32_tile<256>(sl.p, stage, sl.st[in], sl.st[0], (const float*)sl.split,
                                        (const float*)sl.roe, dt, am, sl.st[out], (int)local, sm);
      if (block_or(bad) && threadIdx.x == 0) {
        atomicOr(&d->postag, 1);
        if (sl.use_limiter == 2) atomicOr(&ctl->any_postag, 1);
      }
    } else {
      stage32_ghosts_chunk<256>(sl.p, stage, sl.st[in], sl.st[0], dt, sl.st[out], local - tiles);
    }
    __syncthreads();  // the next item rewrites the tile's shared memory
  }
}

cudaError_t batch_stage32_setup() {
  return cudaFuncSetAttribute(kb_stage32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(Stage32Tile));
}

static int batch_stage32_grid() {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_stage32, 256, sizeof(Stage32Tile));
    grid = (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
  }
  return grid;
}

cudaError_t launch_batch_stage32(const BatchLaunch& b, int stage, int in, int out,
                                 cudaGraphConditionalHandle h_sweep, cudaStream_t s) {
  const int n = b.n_slots;
  const int gs = (n + 127) / 128;
  kb_stage_reset<<<gs, 128, 0, s>>>(b.tab, b.ctl, n);
  kb_alpha_terms32<<<batch_tile_grid(), SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, n, b.ctl, in);
  kb_alpha_final<<<gs, 128, 0, s>>>(b.tab, n, stage);
  kb_stage32<<<batch_stage32_grid(), 256, sizeof(Stage32Tile), s>>>(b.tab, b.s32prefix, n,
                                                                     b.ctl, stage, in, out);
  if (h_sweep) kb_cond_any_postag<<<1, 1, 0, s>>>(h_sweep, b.ctl);
  return cudaGetLastError();
}

cudaError_t launch_batch_alpha(const BatchLaunch& b, int in, cudaStream_t s) {
  kb_alpha<<<batch_tile_grid(), SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, b.n_slots, b.ctl, in);
  return cudaGetLastError();
}

cudaError_t launch_batch_bc(const BatchLaunch& b, int out, cudaStream_t s) {
  kb_bc<<<batch_tile_grid(), SWFD_BLOCK, 0, s>>>(b.tab, b.tprefix, b.n_slots, b.ctl, out);
  return cudaGetLastError();
}

cudaError_t launch_batch_time_advance(const BatchLaunch& b, cudaStream_t s) {
  kb_time_advance<<<(b.n_slots + 127) / 128, 128, 0, s>>>(b.tab, b.ctl, b.n_slots);
  return cudaGetLastError();
}

cudaError_t launch_batch_run_cond(cudaGraphConditionalHandle h, const BatchLaunch& b, int advance,
                                  cudaStream_t s) {
  kb_run_cond<<<1, 1, 0, s>>>(h, b.ctl, advance);
  return cudaGetLastError();
}

}  // namespace swfd
