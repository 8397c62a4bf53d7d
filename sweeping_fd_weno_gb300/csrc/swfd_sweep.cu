// swfd_sweep.cu -- the sweeping post-process: density sweep, u_bar, the
// forward/backward pressure passes with nodal adjustment, and the exit test.
//
// A pass visits the cells of an ordering in sequence; each step may change
// the current cell and its successor, so the visit order is a true data
// dependency.  Positions map to cells arithmetically (snake orderings I and
// II of ex3_vortex_accuracy_2d/main.f90:1211-1270, or the index order of the
// 1D sweep).
#include "swfd_device.cuh"

namespace swfd {

// position -> cell offset; ordering 1 = I (column by column), 2 = II (row by
// row), 0 = 1D index order over -2..n+3
__device__ __forceinline__ int64_t pos_cell(const Geom& g, int ordering, int64_t pos) {
  if (ordering == 0) return pos;  // 1D: position p is cell p-2, offset p
  int i, j;
  if (ordering == 1) {
    j = (int)(pos / g.nx) + 1;
    int t = (int)(pos % g.nx);
    i = (j & 1) ? t + 1 : g.nx - t;
  } else {
    i = (int)(pos / g.ny) + 1;
    int t = (int)(pos % g.ny);
    j = (i & 1) ? t + 1 : g.ny - t;
  }
  return g.at(i, j);
}

__host__ __device__ __forceinline__ int64_t npos(const Geom& g) {
  return g.ndim == 1 ? (int64_t)g.LI : (int64_t)g.nx * g.ny;
}

// pressure as the sweep computes it
// (2D ex3_vortex_accuracy_2d/main.f90:946, 1D ex2_sedov_1d/main.f90:603)
__device__ __forceinline__ double sweep_pres(const Geom& g, double g1, const double* v) {
  if (g.ndim == 1) return g1 * (v[2] - 0.5 * (v[1] * v[1]) / v[0]);
  return g1 * (v[3] - 0.5 * (v[1] * v[1] + v[2] * v[2]) / (v[0]));
}

// nod_lim (ex3_vortex_accuracy_2d/main.f90:846-884; 1D ex2_sedov_1d/main.f90:517-560)
__device__ void nod_lim(const Geom& g, double g1, double eps, const double* v1, const double* v2,
                        const double* vb, double* out, long long& npos_, long long& nneg) {
  double t;
  if (g.ndim == 1) {
    double p1 = g1 * (v1[2] - 0.5 * (v1[1] * v1[1] / v1[0]));
    double p2 = g1 * (v2[2] - 0.5 * (v2[1] * v2[1] / v2[0]));
    if (p2 > eps) {
      t = (p1 - eps) / (p1 - p2);
      ++npos_;
    } else {
      double pb = g1 * (vb[2] - 0.5 * (vb[1] * vb[1] / vb[0]));
      double t_1 = (p1 - eps) / (p1 - pb);
      double d12 = sqrt(dsq(v2[2] - v1[2]) + dsq(v2[1] - v1[1]) + dsq(v2[0] - v1[0]));
      double d1b = sqrt(dsq(vb[2] - v1[2]) + dsq(vb[1] - v1[1]) + dsq(vb[0] - v1[0]));
      t = fmin(t_1 * d1b / d12, 0.25);
      ++nneg;
    }
  } else {
    double p1 = g1 * (v1[3] - 0.5 * (v1[1] * v1[1] + v1[2] * v1[2]) / v1[0]);
    double p2 = g1 * (v2[3] - 0.5 * (v2[1] * v2[1] + v2[2] * v2[2]) / v2[0]);
    if (p2 > eps) {
      t = (p1 - eps) / (p1 - p2);
      ++npos_;
    } else {
      double pb = g1 * (vb[3] - 0.5 * (vb[1] * vb[1] + vb[2] * vb[2]) / vb[0]);
      double t_1 = (p1 - eps) / (p1 - pb);
      double d12 = sqrt(dsq(v2[3] - v1[3]) + dsq(v2[2] - v1[2]) + dsq(v2[1] - v1[1]) +
                        dsq(v2[0] - v1[0]));
      double d1b = sqrt(dsq(vb[3] - v1[3]) + dsq(vb[2] - v1[2]) + dsq(vb[1] - v1[1]) +
                        dsq(vb[0] - v1[0]));
      t = fmin(t_1 * d1b / d12, 0.25);
      ++nneg;
    }
  }
  for (int c = 0; c < g.nc; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}

// ---------------------------------------------------------------------------
// rho_min over the sweep domain (2D interior), ex3_vortex_accuracy_2d/main.f90:1148-1153
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long order_key(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__global__ void k_rho_min(Params p, const double* __restrict__ u, DevScalars* dsc) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)g.nx * g.ny;
  double v = 1e20;
  if (t < n) {
    int i = (int)(t % g.nx) + 1, j = (int)(t / g.nx) + 1;
    v = fmin(u[g.at(i, j)], v);
  }
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMin(&dsc->rho_min_key, order_key(v));
}

cudaError_t launch_rho_min(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(&dsc->rho_min_key, 0xff, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  int64_t n = (int64_t)p.g.nx * p.g.ny;
  k_rho_min<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, u, dsc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// density sweep (2D ordering I, delta = 1d-12: ex3_vortex_accuracy_2d/main.f90:1155-1185;
// 1D over -2..n+3, delta = 1d-13: ex2_sedov_1d/main.f90:742-772).
// All weights are equal, so (w_i/w_next) is exactly 1.
// Sequential reference-order walk in one thread.
// ---------------------------------------------------------------------------
__global__ void k_density_sweep_seq(Params p, double* __restrict__ u) {
  const Geom& g = p.g;
  const int ord = g.ndim == 1 ? 0 : 1;
  const double delta = g.ndim == 1 ? 1e-13 : 1e-12;
  const int64_t N = npos(g);
  double* rho = u;
  // forward
  int64_t c0 = pos_cell(g, ord, 0);
  double cur = rho[c0];
  for (int64_t k = 0; k < N - 1; ++k) {
    int64_t c1 = pos_cell(g, ord, k + 1);
    double nxt = rho[c1];
    if (cur < delta) {
      nxt = nxt + 1.0 * (cur - delta);
      rho[c1] = nxt;
      rho[c0] = delta;
    }
    cur = nxt;
    c0 = c1;
  }
  // backward
  c0 = pos_cell(g, ord, N - 1);
  cur = rho[c0];
  for (int64_t k = N - 1; k >= 1; --k) {
    int64_t c1 = pos_cell(g, ord, k - 1);
    double nxt = rho[c1];
    if (cur < delta) {
      nxt = nxt + 1.0 * (cur - delta);
      rho[c1] = nxt;
      rho[c0] = delta;
    }
    cur = nxt;
    c0 = c1;
  }
}

cudaError_t launch_density_sweep(const Params& p, double* u, cudaStream_t s) {
  k_density_sweep_seq<<<1, 1, 0, s>>>(p, u);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// u_bar: the reference's sequential weighted sums
// (2D j-outer/i-inner, ex3_vortex_accuracy_2d/main.f90:913-920;
//  1D dot_product over -2..n+3, ex2_sedov_1d/main.f90:581-583).
// One lane per component keeps the exact summation order.
// ---------------------------------------------------------------------------
__global__ void k_ubar_seq(Params p, const double* __restrict__ u, DevScalars* dsc) {
  const Geom& g = p.g;
  int c = threadIdx.x;
  if (c >= g.nc) return;
  const double* pl = u + c * g.plane;
  double s = 0.0;
  if (g.ndim == 1) {
    const double w = 1 / ((double)g.nx + 6);
    for (int i = -2; i <= g.nx + 3; ++i) s = s + pl[g.at(i, -2)] * w;
  } else {
    const double w = 1. / ((double)g.nx * (double)g.ny);
    for (int j = 1; j <= g.ny; ++j) {
      const double* row = pl + g.at(0, j);
      for (int i = 1; i <= g.nx; ++i) s = s + w * row[i];
    }
  }
  dsc->ubar[c] = s;
}

cudaError_t launch_ubar(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s) {
  k_ubar_seq<<<1, 32, 0, s>>>(p, u, dsc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// one pressure pass (forward: steps k = 0..N-2 toward k+1; backward: steps
// k = N-1..1 toward k-1), sequential in one thread
// (ex3_vortex_accuracy_2d/main.f90:939-1016; ex2_sedov_1d/main.f90:596-697)
// ---------------------------------------------------------------------------
__global__ void k_pressure_pass_seq(Params p, double* __restrict__ u, int ordering, int forward,
                                    DevScalars* dsc) {
  const Geom& g = p.g;
  if (ordering < 0) ordering = dsc->ordering;
  const int64_t N = npos(g), P = g.plane;
  const double g1 = p.gamma1, eps = p.eps;
  double ub[4];
  for (int c = 0; c < g.nc; ++c) ub[c] = dsc->ubar[c];
  long long np_ = 0, nn = 0;
  int64_t k = forward ? 0 : N - 1;
  const int64_t kend = forward ? N - 1 : 0;
  const int64_t dk = forward ? 1 : -1;
  int64_t c0 = pos_cell(g, ordering, k);
  double vi[4];
  for (int c = 0; c < g.nc; ++c) vi[c] = u[c * P + c0];
  for (; k != kend; k += dk) {
    int64_t c1 = pos_cell(g, ordering, k + dk);
    double vp[4];
    for (int c = 0; c < g.nc; ++c) vp[c] = u[c * P + c1];
    double pres = sweep_pres(g, g1, vi);
    if (pres <= eps || vi[0] <= eps) {
      double vit[4];
      nod_lim(g, g1, eps, vi, vp, ub, vit, np_, nn);
      for (int c = 0; c < g.nc; ++c) {
        double d = vi[c] - vit[c];
        u[c * P + c0] = vit[c];
        vp[c] = vp[c] + 1.0 * (d);
        u[c * P + c1] = vp[c];
      }
    }
    for (int c = 0; c < g.nc; ++c) vi[c] = vp[c];
    c0 = c1;
  }
  dsc->t_pos += np_;
  dsc->t_neg += nn;
}

cudaError_t launch_pressure_pass(const Params& p, double* u, int ordering, int forward,
                                 DevScalars* dsc, cudaStream_t s) {
  k_pressure_pass_seq<<<1, 1, 0, s>>>(p, u, p.g.ndim == 1 ? 0 : ordering, forward, dsc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// exit test: number of cells failing P > eps and rho > eps (ex5: >=) over the
// sweep domain (ex3_vortex_accuracy_2d/main.f90:1106-1119; 1D over -2..n+3)
// ---------------------------------------------------------------------------
__global__ void k_exit_count(Params p, const double* __restrict__ u, DevScalars* dsc) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = npos(g);
  int bad = 0;
  if (t < n) {
    int64_t o;
    if (g.ndim == 1) o = t;
    else o = g.at((int)(t % g.nx) + 1, (int)(t / g.nx) + 1);
    double v[4];
    for (int c = 0; c < g.nc; ++c) v[c] = u[c * g.plane + o];
    double pr = sweep_pres(g, p.gamma1, v);
    if (p.exit_ge) bad = (pr < p.eps) || (v[0] < p.eps);
    else bad = (pr <= p.eps) || (v[0] <= p.eps);
  }
  unsigned m = __ballot_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(&dsc->bad_count, __popc(m));
}

cudaError_t launch_exit_count(const Params& p, const double* u, DevScalars* dsc, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(&dsc->bad_count, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  int64_t n = p.g.ndim == 1 ? (int64_t)p.g.LI : (int64_t)p.g.nx * p.g.ny;
  k_exit_count<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, u, dsc);
  return cudaGetLastError();
}

// ===========================================================================
// Parallel exact passes.
//
// A pass walks positions q = 0..N-1 (q = p forward, q = N-1-p backward); the
// step at q acts only if cell(q) is bad, changes cells q and q+1, and is the
// only step that can touch cell q+1 before the walk reaches it.  A chain is
// a run of consecutive acting steps: it starts at a cell that was bad when
// the pass began, carries the modified cell forward, and ends at the first
// cell that is good on arrival (or at position N-1, which has no step).
// Chains that do not reach the next initially-bad position are independent
// of everything else in the pass, so they run in parallel; a chain that does
// reach it continues with a carried state the start of the next chain did not
// see, and is followed sequentially.  The cells each step reads, writes and
// the arithmetic are those of the sequential walk, so the result is the same
// value for value.
//
// Kernels per pass: flag (bitmask of initially-bad step positions),
// compact (sorted list F), dry run (each F[k] from the original state,
// stopped at F[k+1]: TERM or MERGE), walker (one warp: true roots, and the
// MERGE chains run to their end with writes), write (TERM roots in parallel).
// ===========================================================================

struct SweepScratch {
  uint32_t* bits;    // W = ceil((N-1)/32) words
  int* F;            // flagged positions, sorted
  int* dry_end;      // end position of the dry run
  uint8_t* dry_merge;  // 1: the dry run reached F[k+1]
  uint8_t* root;     // 1: F[k] starts a true TERM chain
  int* counters;     // [0] m, [1] has_merge
};

// kind 0: pressure pass (nodal adjustment); kind 1: density pass
template <int KIND>
struct Chain {
  double s[4];
  __device__ __forceinline__ void load(const Params& p, const double* u, int64_t c) {
    if (KIND == 1) s[0] = u[c];
    else
      for (int k = 0; k < p.g.nc; ++k) s[k] = u[k * p.g.plane + c];
  }
  __device__ __forceinline__ void store(const Params& p, double* u, int64_t c) const {
    if (KIND == 1) u[c] = s[0];
    else
      for (int k = 0; k < p.g.nc; ++k) u[k * p.g.plane + c] = s[k];
  }
  __device__ __forceinline__ bool bad(const Params& p) const {
    if (KIND == 1) return s[0] < (p.g.ndim == 1 ? 1e-13 : 1e-12);
    double pr = sweep_pres(p.g, p.gamma1, s);
    return pr <= p.eps || s[0] <= p.eps;
  }
  // one step: this (cell q) acts on nx (cell q+1); afterwards this holds the
  // final value of cell q and nx the modified value of cell q+1
  __device__ __forceinline__ void step(const Params& p, Chain& nx, const double* ub,
                                       long long& npos_, long long& nneg) {
    if (KIND == 1) {
      const double delta = p.g.ndim == 1 ? 1e-13 : 1e-12;
      nx.s[0] = nx.s[0] + 1.0 * (s[0] - delta);
      s[0] = delta;
    } else {
      double vit[4];
      nod_lim(p.g, p.gamma1, p.eps, s, nx.s, ub, vit, npos_, nneg);
      for (int c = 0; c < p.g.nc; ++c) {
        double d = s[c] - vit[c];
        s[c] = vit[c];
        nx.s[c] = nx.s[c] + 1.0 * (d);
      }
    }
  }
};

__device__ __forceinline__ int64_t walk_cell(const Geom& g, int ordering, int forward, int64_t N,
                                              int64_t q) {
  return pos_cell(g, ordering, forward ? q : N - 1 - q);
}

// Run the chain that starts at q0 (bad on arrival).  stop >= 0 bounds the run:
// reaching position `stop` returns with *merged = 1.  Returns the last
// position the chain modified.
template <int KIND, bool WRITE>
__device__ int64_t run_chain(const Params& p, double* u, int ordering, int forward, int64_t N,
                             int64_t q0, int64_t stop, const double* ub, int* merged,
                             long long& npos_, long long& nneg) {
  const Geom& g = p.g;
  Chain<KIND> cur, nxt;
  int64_t cq = walk_cell(g, ordering, forward, N, q0);
  cur.load(p, u, cq);
  int64_t q = q0;
  *merged = 0;
  for (;;) {
    if (q >= N - 1) {  // the last position takes no step
      if (WRITE) cur.store(p, u, cq);
      return q;
    }
    int64_t cn = walk_cell(g, ordering, forward, N, q + 1);
    nxt.load(p, u, cn);
    cur.step(p, nxt, ub, npos_, nneg);
    if (WRITE) cur.store(p, u, cq);
    ++q;
    cq = cn;
    cur = nxt;
    if (stop >= 0 && q == stop) {
      *merged = 1;
      return q;
    }
    if (!cur.bad(p)) {
      if (WRITE) cur.store(p, u, cq);
      return q;
    }
  }
}

template <int KIND>
__global__ void k_flag_bits(Params p, const double* __restrict__ u, int ordering, int forward,
                            SweepScratch sc, const DevScalars* dsc) {
  const Geom& g = p.g;
  if (ordering < 0) ordering = dsc->ordering;
  const int64_t N = npos(g);
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool b = false;
  if (q < N - 1) {
    Chain<KIND> c;
    c.load(p, u, walk_cell(g, ordering, forward, N, q));
    b = c.bad(p);
  }
  unsigned m = __ballot_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0 && q < N - 1) sc.bits[q >> 5] = m;
}

// single block: bitmask -> sorted positions; counters[0] = m
__global__ void __launch_bounds__(1024) k_compact(int64_t N, SweepScratch sc) {
  __shared__ int part[1024];
  const int64_t W = (N - 1 + 31) / 32;
  const int T = blockDim.x, t = threadIdx.x;
  const int64_t chunk = (W + T - 1) / T;
  const int64_t w0 = t * chunk, w1 = min(W, w0 + chunk);
  int cnt = 0;
  for (int64_t w = w0; w < w1; ++w) cnt += __popc(sc.bits[w]);
  part[t] = cnt;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {  // inclusive scan
    int v = (t >= off) ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int pos = part[t] - cnt;
  for (int64_t w = w0; w < w1; ++w) {
    uint32_t b = sc.bits[w];
    while (b) {
      int i = __ffs(b) - 1;
      b &= b - 1;
      sc.F[pos++] = (int)(w * 32 + i);
    }
  }
  if (t == T - 1) {
    sc.counters[0] = part[T - 1];
    sc.counters[1] = 0;
  }
}

template <int KIND>
__global__ void k_chain_dry(Params p, double* u, int ordering, int forward, SweepScratch sc,
                            const DevScalars* dsc) {
  if (ordering < 0) ordering = dsc->ordering;
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    long long a = 0, b = 0;
    int merged = 0;
    int64_t stop = (k + 1 < m) ? sc.F[k + 1] : -1;
    int64_t e = run_chain<KIND, false>(p, u, ordering, forward, N, sc.F[k], stop, ub, &merged, a,
                                       b);
    sc.dry_end[k] = (int)e;
    sc.dry_merge[k] = (uint8_t)merged;
    sc.root[k] = 0;
    if (merged) atomicOr(&sc.counters[1], 1);
  }
}

// one warp: resolve true roots; run MERGE chains to their end with writes
template <int KIND>
__global__ void k_chain_walk(Params p, double* u, int ordering, int forward, SweepScratch sc,
                             DevScalars* dsc) {
  if (sc.counters[1] == 0) return;  // no chain reaches the next flagged cell
  if (ordering < 0) ordering = dsc->ordering;
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  const int lane = threadIdx.x;
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
  long long npos_ = 0, nneg = 0;
  int64_t covered = -1;
  int base = 0;
  while (base < m) {
    int k = base + lane;
    bool valid = k < m;
    int64_t f = valid ? sc.F[k] : INT64_MAX;
    bool mg = valid && sc.dry_merge[k];
    bool live = valid && f > covered;
    unsigned mm = __ballot_sync(0xffffffffu, live && mg);
    int first = mm ? __ffs(mm) - 1 : 32;
    if (live && !mg && lane < first) sc.root[k] = 1;
    if (first == 32) {
      base += 32;
      continue;
    }
    int64_t e = 0;
    if (lane == first) {
      int merged;
      e = run_chain<KIND, true>(p, u, ordering, forward, N, f, -1, ub, &merged, npos_, nneg);
    }
    covered = __shfl_sync(0xffffffffu, e, first);
    base += first + 1;
  }
  if (KIND == 0 && (npos_ | nneg)) {  // each lane adds the chains it ran
    atomicAdd((unsigned long long*)&dsc->t_pos, (unsigned long long)npos_);
    atomicAdd((unsigned long long*)&dsc->t_neg, (unsigned long long)nneg);
  }
}

template <int KIND>
__global__ void k_chain_write(Params p, double* u, int ordering, int forward, SweepScratch sc,
                              DevScalars* dsc) {
  if (ordering < 0) ordering = dsc->ordering;
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  const bool all_roots = sc.counters[1] == 0;
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
  long long npos_ = 0, nneg = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    if (!(all_roots || sc.root[k])) continue;
    int merged;
    run_chain<KIND, true>(p, u, ordering, forward, N, sc.F[k], -1, ub, &merged, npos_, nneg);
  }
  if (KIND == 0 && (npos_ | nneg)) {
    atomicAdd((unsigned long long*)&dsc->t_pos, (unsigned long long)npos_);
    atomicAdd((unsigned long long*)&dsc->t_neg, (unsigned long long)nneg);
  }
}

size_t sweep_scratch_bytes(const Params& p) {
  const int64_t N = npos(p.g);
  const int64_t W = (N + 31) / 32 + 1;
  return W * 4 + N * 4 * 2 + N * 2 + 64 + 256;
}

static SweepScratch carve(void* base, const Params& p) {
  const int64_t N = npos(p.g);
  const int64_t W = (N + 31) / 32 + 1;
  char* c = (char*)base;
  SweepScratch s;
  s.counters = (int*)c;
  c += 64;
  s.bits = (uint32_t*)c;
  c += W * 4;
  s.F = (int*)c;
  c += N * 4;
  s.dry_end = (int*)c;
  c += N * 4;
  s.dry_merge = (uint8_t*)c;
  c += N;
  s.root = (uint8_t*)c;
  return s;
}

template <int KIND>
static cudaError_t pass_parallel(const Params& p, double* u, int ordering, int forward,
                                 void* scratch, DevScalars* dsc, cudaStream_t s, int* nlaunch) {
  const int64_t N = npos(p.g);
  SweepScratch sc = carve(scratch, p);
  const int ord = p.g.ndim == 1 ? 0 : ordering;
  k_flag_bits<KIND><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(p, u, ord, forward, sc, dsc);
  k_compact<<<1, 1024, 0, s>>>(N, sc);
  const int grid = 4 * 152;
  k_chain_dry<KIND><<<grid, 128, 0, s>>>(p, u, ord, forward, sc, dsc);
  k_chain_walk<KIND><<<1, 32, 0, s>>>(p, u, ord, forward, sc, dsc);
  k_chain_write<KIND><<<grid, 128, 0, s>>>(p, u, ord, forward, sc, dsc);
  *nlaunch += 5;
  return cudaGetLastError();
}

cudaError_t launch_pressure_pass_par(const Params& p, double* u, int ordering, int forward,
                                     void* scratch, DevScalars* dsc, cudaStream_t s, int* nlaunch) {
  return pass_parallel<0>(p, u, ordering, forward, scratch, dsc, s, nlaunch);
}

cudaError_t launch_density_sweep_par(const Params& p, double* u, void* scratch, cudaStream_t s,
                                     int* nlaunch) {
  cudaError_t e = pass_parallel<1>(p, u, 1, 1, scratch, nullptr, s, nlaunch);
  if (e != cudaSuccess) return e;
  return pass_parallel<1>(p, u, 1, 0, scratch, nullptr, s, nlaunch);
}

}  // namespace swfd
