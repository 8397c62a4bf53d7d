// swfd_sweep.cu -- the sweeping post-process: density sweep, u_bar, the
// forward/backward pressure passes with nodal adjustment, and the exit test.
//
// A pass visits the cells of an ordering in sequence; each step may change
// the current cell and its successor, so the visit order is a true data
// dependency.  Positions map to cells arithmetically (snake orderings I and
// II of ex3_vortex_accuracy_2d/main.f90:1211-1270, or the index order of the
// 1D sweep).
#include "swfd_sweep.cuh"

namespace swfd {

// ---------------------------------------------------------------------------
// rho_min over the sweep domain (2D interior), ex3_vortex_accuracy_2d/main.f90:1148-1153
// ---------------------------------------------------------------------------
__global__ void k_rho_min(Params p, const double* __restrict__ u, DevScalars* dsc) {
  const Geom& g = p.g;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t n = (int64_t)g.nx * g.ny;
  double v = 1e20;
  if (t < n) {
    int i = ((int)t % g.nx) + 1, j = ((int)t / g.nx) + 1;
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
// The sum is a chain of dependent FP64 additions in the reference's order,
// and a dependent FP64 addition on GB300 takes about 66 cycles.  The chain is
// evaluated exactly without it: while the exact value s + p of a step stays
// inside the binade [2^E, 2^(E+1)) of the running sum s = M * u (u = 2^(E-52),
// M an integer in [2^52, 2^53]), the rounded result is (M + rne(p / u)) * u,
// with rne the round-to-nearest of an integer-plus-fraction, so a run of such
// steps is an integer prefix sum (done by the whole block in parallel).  The
// first step of a window that leaves the binade, is a rounding tie (whose
// result depends on the parity of the running sum), or meets a zero,
// subnormal or non-finite value is done as one hardware addition, and the
// integer path resumes after it.  Every step therefore rounds exactly as the
// sequential loop does.
constexpr int SUM_THREADS = 256;
constexpr int SUM_PER_THREAD = 8;
constexpr int SUM_WINDOW = SUM_THREADS * SUM_PER_THREAD;

// The batched engine's form (the single-instance sweep uses swfd_ubar.cu):
// s = 0; for m = 0..n-1: s = s + term(m)  (term(m) the FP64 product of the
// reference), evaluated by one block of SUM_THREADS threads; every thread
// returns s
template <class Term>
__device__ double seq_sum_block(int n, Term term) {
  __shared__ unsigned long long warp_tot[SUM_THREADS / 32];
  __shared__ int first_bad;
  __shared__ double s_sh;
  __shared__ int pos_sh;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  double s = 0.0;
  int pos = 0;
  while (pos < n) {
    const unsigned long long sb = (unsigned long long)__double_as_longlong(s);
    const int eb = (int)((sb >> 52) & 0x7ff);
    if (eb == 0 || eb == 0x7ff) {  // zero, subnormal or non-finite sum: one hardware step
      s = s + term(pos);
      ++pos;
      continue;
    }
    const int neg_s = (int)(sb >> 63);
    const long long M = (long long)((sb & 0xfffffffffffffull) | (1ull << 52));
    const int base = pos + tid * SUM_PER_THREAD;
    long long fl[SUM_PER_THREAD], r[SUM_PER_THREAD];
    int bad[SUM_PER_THREAD];
    unsigned long long tsum = 0;
#pragma unroll
    for (int e = 0; e < SUM_PER_THREAD; ++e) {
      const int m = base + e;
      if (m < n) {
        sum_classify(term(m), neg_s, eb, fl[e], r[e], bad[e]);
      } else {
        fl[e] = r[e] = 0;
        bad[e] = 2;  // past the end
      }
      tsum += (unsigned long long)r[e];
    }
    // block-exclusive prefix of the per-thread sums (wrapping arithmetic: the
    // values up to the first bad element are exact)
    unsigned long long incl = tsum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned long long v = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += v;
    }
    if (lane == 31) warp_tot[wid] = incl;
    if (tid == 0) first_bad = INT_MAX;
    __syncthreads();
    unsigned long long R = incl - tsum;
    for (int k = 0; k < wid; ++k) R += warp_tot[k];
    int myfirst = INT_MAX;
#pragma unroll
    for (int e = 0; e < SUM_PER_THREAD; ++e) {
      if (myfirst != INT_MAX) break;
      const long long a = M + (long long)R + fl[e];
      if (bad[e] || a < (1ll << 52) || a > (1ll << 53) - 1) {
        myfirst = base + e;
      } else {
        R += (unsigned long long)r[e];
      }
    }
    if (myfirst != INT_MAX) atomicMin(&first_bad, myfirst);
    __syncthreads();
    const int q = first_bad;
    const bool writer = (q == INT_MAX) ? (tid == SUM_THREADS - 1) : (myfirst == q);
    if (writer) {
      // the sum after the integer run, M + R in units of u (in [2^52, 2^53])
      const unsigned long long val = (unsigned long long)(M + (long long)R);
      unsigned long long bits = (val == (1ull << 53))
                                    ? ((unsigned long long)(eb + 1) << 52)
                                    : (((unsigned long long)eb << 52) | (val - (1ull << 52)));
      bits |= (unsigned long long)neg_s << 63;
      double sn = __longlong_as_double((long long)bits);
      int np;
      if (q == INT_MAX) {
        np = pos + SUM_WINDOW;
      } else if (q < n) {
        sn = sn + term(q);  // the step the integer path does not take
        np = q + 1;
      } else {
        np = n;
      }
      s_sh = sn;
      pos_sh = np;
    }
    __syncthreads();
    s = s_sh;
    pos = pos_sh;
    __syncthreads();
  }
  return s;
}

// u_bar of one component (blockIdx.x): 2D weights 1/(nx*ny) over the interior
// in j-outer/i-inner order, 1D 1/(n+6) over -2..n+3
__device__ void ubar_component(const Geom& g, const double* __restrict__ u, int c, double* out) {
  const double* pl = u + c * g.plane;
  double s;
  if (g.ndim == 1) {
    const double w = 1 / ((double)g.nx + 6);
    s = seq_sum_block(g.nx + 6, [&](int m) { return pl[m] * w; });
  } else {
    const double w = 1. / ((double)g.nx * (double)g.ny);
    const int nx = g.nx;
    s = seq_sum_block(g.nx * g.ny, [&](int m) { return w * pl[g.at(m % nx + 1, m / nx + 1)]; });
  }
  if (threadIdx.x == 0) out[c] = s;
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
      const double pp = sweep_pres(g, g1, vp);
      nod_lim(g, g1, eps, vi, vp, ub, vit, np_, nn);
      for (int c = 0; c < g.nc; ++c) {
        double d = vi[c] - vit[c];
        u[c * P + c0] = vit[c];
        vp[c] = vp[c] + 1.0 * (d);
        u[c * P + c1] = vp[c];
      }
      // ex6 (ex6_shock_diffraction/main.f90:1413-1423, ordering-I passes)
      if (p.sweep_check && ordering == 1 &&
          pres + pp > sweep_pres(g, g1, vit) + sweep_pres(g, g1, vp) + eps)
        dsc->error |= ERR_BIT_CHECK;
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
    else o = g.at(((int)t % g.nx) + 1, ((int)t / g.nx) + 1);
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
// stopped at F[k+1]: TERM or MERGE), cluster walk (one thread per cluster of
// MERGE chains ending in a TERM chain, with writes), fix-up (one warp: counts,
// and the rare cluster walk that reached the next cluster's first position).
// The batched engine runs the earlier form: dry run, one warp following the
// MERGE chains in sequence, and the TERM roots written in parallel.
// ===========================================================================

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

size_t sweep_scratch_bytes(const Params& p) { return sweep_scratch_bytes_impl(p); }
size_t sweep_cluster_bytes(const Params& p) { return cluster_scratch_bytes(p); }

// ---------------------------------------------------------------------------
// Cluster-parallel pass (single-instance path): dry runs as above that also
// keep each flagged cell's pass-start value, one thread per cluster walking
// its chains with writes, and one warp that sums the counts and, when a
// cluster's walk reached the next cluster's first position, undoes the later
// clusters and finishes the pass sequentially.  Values and counts are those
// of the sequential walk.
// ---------------------------------------------------------------------------
template <int KIND>
__device__ __forceinline__ int nc_of(const Params& p) { return KIND == 1 ? 1 : p.g.nc; }

template <int KIND>
__global__ void k_cl_dry(Params p, double* u, int ordering, int forward, SweepScratch sc,
                         ClusterScratch cs, const DevScalars* dsc) {
  if (ordering < 0) ordering = dsc->ordering;
  const Geom& g = p.g;
  const int64_t N = npos(g);
  const int m = sc.counters[0];
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const int64_t cell = walk_cell(g, ordering, forward, N, sc.F[k]);
    for (int c = 0; c < nc_of<KIND>(p); ++c) cs.orig[(int64_t)k * 4 + c] = u[c * g.plane + cell];
    long long a = 0, b = 0;
    int merged = 0;
    int64_t stop = (k + 1 < m) ? sc.F[k + 1] : -1;
    run_chain<KIND, false>(p, u, ordering, forward, N, sc.F[k], stop, ub, &merged, a, b);
    sc.dry_merge[k] = (uint8_t)merged;
  }
}

template <int KIND>
__device__ __forceinline__ void bk_save(const Params& p, const double* u, const ClusterScratch& cs,
                                        int64_t N, int64_t pos, int64_t cell) {
  for (int c = 0; c < nc_of<KIND>(p); ++c) cs.backup[c * N + pos] = u[c * p.g.plane + cell];
}

template <int KIND>
__global__ void k_cl_run(Params p, double* u, int ordering, int forward, SweepScratch sc,
                         ClusterScratch cs, const DevScalars* dsc) {
  if (ordering < 0) ordering = dsc->ordering;
  const Geom& g = p.g;
  const int64_t N = npos(g);
  const int m = sc.counters[0];
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
  const bool check = KIND == 0 && p.sweep_check && ordering == 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    if (k > 0 && sc.dry_merge[k - 1]) {
      cs.flag[k] = 0;  // inside a cluster
      continue;
    }
    int k1 = k;  // the cluster's last chain
    while (k1 < m - 1 && sc.dry_merge[k1]) ++k1;
    const int kn = k1 + 1;
    const int64_t stop = kn < m ? sc.F[kn] : -1;
    long long np_ = 0, nn = 0;
    int fail = 0;
    uint8_t fl = 1;
    int64_t covered = -1, bk = sc.F[k];
    for (int j = k; j <= k1 && fl == 1; ++j) {
      const int64_t q0 = sc.F[j];
      if (q0 <= covered) continue;  // absorbed by the previous chain
      for (; bk <= q0; ++bk) bk_save<KIND>(p, u, cs, N, bk, walk_cell(g, ordering, forward, N, bk));
      Chain<KIND> cur, nxt;
      int64_t q = q0, cq = walk_cell(g, ordering, forward, N, q0);
      cur.load(p, u, cq);
      for (;;) {
        if (q >= N - 1) {  // the last position takes no step
          cur.store(p, u, cq);
          covered = q;
          break;
        }
        int64_t cn = 0;
        if (q + 1 == stop) {  // the next cluster's cell, as it was when the pass began
          for (int c = 0; c < nc_of<KIND>(p); ++c) nxt.s[c] = cs.orig[(int64_t)kn * 4 + c];
        } else {
          cn = walk_cell(g, ordering, forward, N, q + 1);
          for (; bk <= q + 1; ++bk) bk_save<KIND>(p, u, cs, N, bk, walk_cell(g, ordering, forward, N, bk));
          nxt.load(p, u, cn);
        }
        cur.step(p, nxt, ub, np_, nn, check ? &fail : nullptr);
        cur.store(p, u, cq);
        ++q;
        if (q == stop) {  // spill: the carried value of the next cluster's first cell
          for (int c = 0; c < nc_of<KIND>(p); ++c) cs.carry[(int64_t)k * 4 + c] = nxt.s[c];
          fl = 2;
          covered = q - 1;
          break;
        }
        cq = cn;
        cur = nxt;
        if (!cur.bad(p)) {
          cur.store(p, u, cq);
          covered = q;
          break;
        }
      }
    }
    cs.end[k] = (int)covered;
    cs.next[k] = kn;
    cs.cnt[2 * (int64_t)k] = np_;
    cs.cnt[2 * (int64_t)k + 1] = nn;
    cs.flag[k] = fl | (fail ? 4 : 0);
  }
}

template <int KIND>
__global__ void k_cl_fix(Params p, double* u, int ordering, int forward, SweepScratch sc,
                         ClusterScratch cs, DevScalars* dsc) {
  if (ordering < 0) ordering = dsc->ordering;
  const Geom& g = p.g;
  const int64_t N = npos(g);
  const int m = sc.counters[0];
  const int lane = threadIdx.x;
  // the first cluster whose walk stopped at the next cluster's first position
  int first = INT_MAX;
  for (int k = lane; k < m; k += 32)
    if (cs.flag[k] & 2) {
      first = k;
      break;
    }
  for (int off = 16; off > 0; off >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, off));
  long long np_ = 0, nn = 0;
  int fail = 0;
  for (int k = lane; k < m && k <= first; k += 32)
    if (cs.flag[k]) {
      np_ += cs.cnt[2 * (int64_t)k];
      nn += cs.cnt[2 * (int64_t)k + 1];
      fail |= cs.flag[k] & 4;
    }
  if (first != INT_MAX) {
    // undo the clusters after it (disjoint position ranges, one lane each)
    for (int k = first + 1 + lane; k < m; k += 32) {
      if (!cs.flag[k]) continue;
      for (int64_t q = sc.F[k]; q <= cs.end[k]; ++q) {
        const int64_t cell = walk_cell(g, ordering, forward, N, q);
        for (int c = 0; c < nc_of<KIND>(p); ++c) u[c * g.plane + cell] = cs.backup[c * N + q];
      }
    }
    __syncwarp();
    if (lane == 0) {
      double ub[4] = {0, 0, 0, 0};
      if (KIND == 0)
        for (int c = 0; c < 4; ++c) ub[c] = dsc->ubar[c];
      int* chk = (KIND == 0 && p.sweep_check && ordering == 1) ? &fail : nullptr;
      // the spilled chain from the next cluster's first position with its carried value
      const int kn = cs.next[first];
      int64_t q = sc.F[kn], cq = walk_cell(g, ordering, forward, N, q);
      Chain<KIND> cur, nxt;
      for (int c = 0; c < nc_of<KIND>(p); ++c) cur.s[c] = cs.carry[(int64_t)first * 4 + c];
      for (;;) {
        if (!cur.bad(p) || q >= N - 1) {
          cur.store(p, u, cq);
          break;
        }
        const int64_t cn = walk_cell(g, ordering, forward, N, q + 1);
        nxt.load(p, u, cn);
        cur.step(p, nxt, ub, np_, nn, chk);
        cur.store(p, u, cq);
        ++q;
        cq = cn;
        cur = nxt;
      }
      // then every later flagged position the walk has not reached, in order
      int64_t covered = q;
      for (int j = kn + 1; j < m; ++j) {
        if (sc.F[j] <= covered) continue;
        int merged;
        covered = run_chain<KIND, true>(p, u, ordering, forward, N, sc.F[j], -1, ub, &merged, np_,
                                        nn, chk);
      }
    }
  }
  if constexpr (KIND == 0) {
    for (int off = 16; off > 0; off >>= 1) {
      np_ += __shfl_xor_sync(0xffffffffu, np_, off);
      nn += __shfl_xor_sync(0xffffffffu, nn, off);
      fail |= __shfl_xor_sync(0xffffffffu, fail, off);
    }
    if (lane == 0) {
      if (fail) atomicOr(&dsc->error, ERR_BIT_CHECK);
      if (np_ | nn) {
        atomicAdd((unsigned long long*)&dsc->t_pos, (unsigned long long)np_);
        atomicAdd((unsigned long long*)&dsc->t_neg, (unsigned long long)nn);
      }
    }
  }
}

template <int KIND>
static cudaError_t pass_parallel(const Params& p, double* u, int ordering, int forward,
                                 void* scratch, void* cluster, DevScalars* dsc, cudaStream_t s,
                                 int* nlaunch) {
  const int64_t N = npos(p.g);
  SweepScratch sc = carve(scratch, p);
  ClusterScratch cs = carve_cluster(cluster, p);
  const int ord = p.g.ndim == 1 ? 0 : ordering;
  k_flag_bits<KIND><<<(unsigned)((N + 255) / 256), 256, 0, s>>>(p, u, ord, forward, sc, dsc);
  k_compact<<<1, 1024, 0, s>>>(N, sc);
  const int grid = 4 * 152;
  k_cl_dry<KIND><<<grid, 128, 0, s>>>(p, u, ord, forward, sc, cs, dsc);
  k_cl_run<KIND><<<grid, 128, 0, s>>>(p, u, ord, forward, sc, cs, dsc);
  k_cl_fix<KIND><<<1, 32, 0, s>>>(p, u, ord, forward, sc, cs, dsc);
  *nlaunch += 5;
  return cudaGetLastError();
}

cudaError_t launch_pressure_pass_par(const Params& p, double* u, int ordering, int forward,
                                     void* scratch, void* cluster, DevScalars* dsc,
                                     cudaStream_t s, int* nlaunch) {
  return pass_parallel<0>(p, u, ordering, forward, scratch, cluster, dsc, s, nlaunch);
}

cudaError_t launch_density_sweep_par(const Params& p, double* u, void* scratch, void* cluster,
                                     cudaStream_t s, int* nlaunch) {
  cudaError_t e = pass_parallel<1>(p, u, 1, 1, scratch, cluster, nullptr, s, nlaunch);
  if (e != cudaSuccess) return e;
  return pass_parallel<1>(p, u, 1, 0, scratch, cluster, nullptr, s, nlaunch);
}

}  // namespace swfd

// ===========================================================================
// Batched sweep kernels: blockIdx.y indexes the slot table; a slot takes part
// while its `sweeping` flag (pressure passes) or `dens_active` flag (density
// passes) is set.  Each slot's passes are exactly the single-instance ones,
// on its stage output buffer st[out].
// ===========================================================================
namespace swfd {

__device__ __forceinline__ bool slot_in(const BatchSlot& sl, int kind) {
  if (!sl.active) return false;
  return kind == 1 ? sl.dsc->dens_active != 0 : sl.dsc->sweeping != 0;
}

// per slot: does this stage sweep?  (use_limiter == 2 and postag)
__global__ void kb_sweep_start(BatchSlot* __restrict__ tab, BatchCtl* ctl, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) ctl->n_sweeping = 0;
  if (s >= n || !tab[s].active) return;
  DevScalars* d = tab[s].dsc;
  d->sweeping = (tab[s].use_limiter == 2 && d->postag) ? 1 : 0;
  d->dens_active = 0;
  d->rho_min_key = ~0ull;
}

// rho_min over the interior (ex3_vortex_accuracy_2d/main.f90:1148-1153)
__global__ void kb_rho_min(const BatchSlot* __restrict__ tab, int out) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, 0)) return;
  const Geom& g = sl.p.g;
  const double* u = sl.st[out];
  const int64_t n = (int64_t)g.nx * g.ny;
  double v = 1e20;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    v = fmin(u[g.at(((int)t % g.nx) + 1, ((int)t / g.nx) + 1)], v);
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMin(&sl.dsc->rho_min_key, order_key(v));
}

__device__ __forceinline__ double decode_key_b(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

// IF rho_min < 1d-12 (:1156); den_count (:1187)
__global__ void kb_density_decide(const BatchSlot* __restrict__ tab, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !slot_in(tab[s], 0)) return;
  DevScalars* d = tab[s].dsc;
  d->dens_active = decode_key_b(d->rho_min_key) < 1e-12 ? 1 : 0;
  if (d->dens_active) d->den_count++;
}

// ordering: 1 (density, ordering I) or -1 (pressure, the slot's dsc->ordering)
template <int KIND>
__global__ void kb_flag(const BatchSlot* __restrict__ tab, int out, int ordering, int forward) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, KIND)) return;
  const Params& p = sl.p;
  const Geom& g = p.g;
  const int ord = ordering >= 0 ? ordering : sl.dsc->ordering;
  const double* u = sl.st[out];
  SweepScratch sc = carve(sl.sweep_scratch, p);
  const int64_t N = npos(g);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;  // a multiple of 32
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < N - 1; base += stride) {
    int64_t q = base + threadIdx.x;
    bool b = false;
    if (q < N - 1) {
      Chain<KIND> c;
      c.load(p, u, walk_cell(g, ord, forward, N, q));
      b = c.bad(p);
    }
    unsigned m = __ballot_sync(0xffffffffu, b);
    if ((threadIdx.x & 31) == 0 && q < N - 1) sc.bits[q >> 5] = m;
  }
}

template <int KIND>
__global__ void __launch_bounds__(1024) kb_compact(const BatchSlot* __restrict__ tab) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, KIND)) return;
  __shared__ int part[1024];
  SweepScratch sc = carve(sl.sweep_scratch, sl.p);
  const int64_t N = npos(sl.p.g);
  const int64_t W = (N - 1 + 31) / 32;
  const int T = blockDim.x, t = threadIdx.x;
  const int64_t chunk = (W + T - 1) / T;
  const int64_t w0 = t * chunk, w1 = min(W, w0 + chunk);
  int cnt = 0;
  for (int64_t w = w0; w < w1; ++w) cnt += __popc(sc.bits[w]);
  part[t] = cnt;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
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
__global__ void kb_dry(const BatchSlot* __restrict__ tab, int out, int ordering, int forward) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, KIND)) return;
  const Params& p = sl.p;
  const int ord = ordering >= 0 ? ordering : sl.dsc->ordering;
  double* u = sl.st[out];
  SweepScratch sc = carve(sl.sweep_scratch, p);
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = sl.dsc->ubar[c];
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    long long a = 0, b = 0;
    int merged = 0;
    int64_t stop = (k + 1 < m) ? sc.F[k + 1] : -1;
    int64_t e = run_chain<KIND, false>(p, u, ord, forward, N, sc.F[k], stop, ub, &merged, a, b);
    sc.dry_end[k] = (int)e;
    sc.dry_merge[k] = (uint8_t)merged;
    sc.root[k] = 0;
    if (merged) atomicOr(&sc.counters[1], 1);
  }
}

template <int KIND>
__global__ void kb_walk(const BatchSlot* __restrict__ tab, int out, int ordering, int forward) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, KIND)) return;
  const Params& p = sl.p;
  SweepScratch sc = carve(sl.sweep_scratch, p);
  if (sc.counters[1] == 0) return;
  const int ord = ordering >= 0 ? ordering : sl.dsc->ordering;
  double* u = sl.st[out];
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  const int lane = threadIdx.x;
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = sl.dsc->ubar[c];
  long long npos_ = 0, nneg = 0;
  int fail = 0;
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
      e = run_chain<KIND, true>(p, u, ord, forward, N, f, -1, ub, &merged, npos_, nneg, &fail);
    }
    covered = __shfl_sync(0xffffffffu, e, first);
    base += first + 1;
  }
  if (KIND == 0 && fail) atomicOr(&sl.dsc->error, ERR_BIT_CHECK);
  if (KIND == 0 && (npos_ | nneg)) {
    atomicAdd((unsigned long long*)&sl.dsc->t_pos, (unsigned long long)npos_);
    atomicAdd((unsigned long long*)&sl.dsc->t_neg, (unsigned long long)nneg);
  }
}

template <int KIND>
__global__ void kb_write(const BatchSlot* __restrict__ tab, int out, int ordering, int forward) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, KIND)) return;
  const Params& p = sl.p;
  const int ord = ordering >= 0 ? ordering : sl.dsc->ordering;
  double* u = sl.st[out];
  SweepScratch sc = carve(sl.sweep_scratch, p);
  const int64_t N = npos(p.g);
  const int m = sc.counters[0];
  const bool all_roots = sc.counters[1] == 0;
  double ub[4] = {0, 0, 0, 0};
  if (KIND == 0)
    for (int c = 0; c < 4; ++c) ub[c] = sl.dsc->ubar[c];
  long long npos_ = 0, nneg = 0;
  int fail = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    if (!(all_roots || sc.root[k])) continue;
    int merged;
    run_chain<KIND, true>(p, u, ord, forward, N, sc.F[k], -1, ub, &merged, npos_, nneg, &fail);
  }
  if (KIND == 0 && fail) atomicOr(&sl.dsc->error, ERR_BIT_CHECK);
  if (KIND == 0 && (npos_ | nneg)) {
    atomicAdd((unsigned long long*)&sl.dsc->t_pos, (unsigned long long)npos_);
    atomicAdd((unsigned long long*)&sl.dsc->t_neg, (unsigned long long)nneg);
  }
}

// u_bar: the reference's sequential sums (one thread per component), or a
// deterministic block tree sum (ubar_tree)
__global__ void kb_ubar(const BatchSlot* __restrict__ tab, int out, int tree) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, 0)) return;
  const Geom& g = sl.p.g;
  const double* u = sl.st[out];
  const double w = 1. / ((double)g.nx * (double)g.ny);
  if (!tree) {
    if ((int)blockIdx.x < g.nc) ubar_component(g, u, blockIdx.x, sl.dsc->ubar);
    return;
  }
  if (blockIdx.x != 0) return;
  __shared__ double red[4][256];
  double acc[4] = {0, 0, 0, 0};
  const int64_t n = (int64_t)g.nx * g.ny;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int64_t o = g.at(((int)t % g.nx) + 1, ((int)t / g.nx) + 1);
    for (int c = 0; c < 4; ++c) acc[c] = acc[c] + w * u[c * g.plane + o];
  }
  for (int c = 0; c < 4; ++c) red[c][threadIdx.x] = acc[c];
  __syncthreads();
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off)
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 4; ++c) sl.dsc->ubar[c] = red[c][0];
}

// sweep_lim set-up (:928-930; ex4's P(u_bar) stop :1447-1454)
__global__ void kb_sweep_begin(BatchSlot* __restrict__ tab, BatchCtl* ctl, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !slot_in(tab[s], 0)) return;
  DevScalars* d = tab[s].dsc;
  const Params& p = tab[s].p;
  if (p.stop_sweep) {
    const double* ub = d->ubar;
    if (p.gamma1 * (ub[3] - 0.5 * (ub[1] * ub[1] + ub[2] * ub[2]) / ub[0]) <= 0.) {
      d->error |= ERR_BIT_PUBAR;
      d->sweeping = 0;
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
  atomicAdd(&ctl->n_sweeping, 1);
}

__global__ void kb_q_begin(const BatchSlot* __restrict__ tab, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !slot_in(tab[s], 0)) return;
  DevScalars* d = tab[s].dsc;
  int q = ++d->q;
  d->ordering = (q & 1) ? 1 : 2;
  d->bad_count = 0;
}

// exit test cells (:1106-1119; `>=` in ex5)
__global__ void kb_exit_count(const BatchSlot* __restrict__ tab, int out) {
  const BatchSlot& sl = tab[blockIdx.y];
  if (!slot_in(sl, 0)) return;
  const Params& p = sl.p;
  const Geom& g = p.g;
  const double* u = sl.st[out];
  const int64_t n = (int64_t)g.nx * g.ny;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = base + threadIdx.x;
    int bad = 0;
    if (t < n) {
      const int64_t o = g.at(((int)t % g.nx) + 1, ((int)t / g.nx) + 1);
      double v[4];
      for (int c = 0; c < 4; ++c) v[c] = u[c * g.plane + o];
      double pr = sweep_pres(g, p.gamma1, v);
      if (p.exit_ge) bad = (pr < p.eps) || (v[0] < p.eps);
      else bad = (pr <= p.eps) || (v[0] <= p.eps);
    }
    unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(&sl.dsc->bad_count, __popc(m));
  }
}

// end of iteration q: pre_count, exit test, tracks (:1116-1129)
__global__ void kb_q_end(BatchSlot* __restrict__ tab, BatchCtl* ctl, int n) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !slot_in(tab[s], 0)) return;
  DevScalars* d = tab[s].dsc;
  d->pre_count++;
  bool stop = false;
  if (d->error & ERR_BIT_CHECK) {  // ex6 stopped inside the passes
    stop = true;
  } else if (d->bad_count == 0) {
    long long k = d->sweep_count - 1;
    if (k >= 0 && k < d->track_cap) {
      d->tracks[k] = d->q;
      d->tracks[d->track_cap + k] = (int)d->t_neg;
      d->tracks[2 * d->track_cap + k] = (int)d->t_pos;
    }
    stop = true;
  } else if (d->q >= tab[s].swp_num) {
    d->fail_count++;
    if (tab[s].stop_on_fail) d->error |= ERR_BIT_NOCONV;
    stop = true;
  }
  if (stop) {
    d->sweeping = 0;
    atomicSub(&ctl->n_sweeping, 1);
  }
}

__global__ void kb_q_cond(cudaGraphConditionalHandle h, BatchCtl* ctl) {
  set_cond(h, &ctl->cond, ctl->n_sweeping > 0 ? 1u : 0u);
}

static int bgx(const BatchLaunch& b) {
  long long want = (4096 + b.n_slots - 1) / b.n_slots;
  long long cap = (b.max_cell + 255) / 256;
  long long x = want < 64 ? 64 : want;
  if (x > cap) x = cap;
  return (int)(x < 1 ? 1 : x);
}

template <int KIND>
static void batch_pass(const BatchLaunch& b, int out, int ordering, int forward, cudaStream_t s) {
  const int n = b.n_slots;
  kb_flag<KIND><<<dim3(bgx(b), n), 256, 0, s>>>(b.tab, out, ordering, forward);
  kb_compact<KIND><<<dim3(1, n), 1024, 0, s>>>(b.tab);
  kb_dry<KIND><<<dim3(4, n), 128, 0, s>>>(b.tab, out, ordering, forward);
  kb_walk<KIND><<<dim3(1, n), 32, 0, s>>>(b.tab, out, ordering, forward);
  kb_write<KIND><<<dim3(4, n), 128, 0, s>>>(b.tab, out, ordering, forward);
}

cudaError_t launch_batch_sweep_head(const BatchLaunch& b, int out, cudaStream_t s) {
  const int n = b.n_slots, gs = (n + 127) / 128;
  kb_sweep_start<<<gs, 128, 0, s>>>(b.tab, b.ctl, n);
  kb_rho_min<<<dim3(bgx(b), n), 256, 0, s>>>(b.tab, out);
  kb_density_decide<<<gs, 128, 0, s>>>(b.tab, n);
  batch_pass<1>(b, out, 1, 1, s);
  batch_pass<1>(b, out, 1, 0, s);
  kb_ubar<<<dim3(4, n), SUM_THREADS, 0, s>>>(b.tab, out, b.ubar_tree);
  kb_sweep_begin<<<gs, 128, 0, s>>>(b.tab, b.ctl, n);
  return cudaGetLastError();
}

cudaError_t launch_batch_sweep_iter(const BatchLaunch& b, int out, cudaGraphConditionalHandle h,
                                    cudaStream_t s) {
  const int n = b.n_slots, gs = (n + 127) / 128;
  kb_q_begin<<<gs, 128, 0, s>>>(b.tab, n);
  batch_pass<0>(b, out, -1, 1, s);
  batch_pass<0>(b, out, -1, 0, s);
  kb_exit_count<<<dim3(bgx(b), n), 256, 0, s>>>(b.tab, out);
  kb_q_end<<<gs, 128, 0, s>>>(b.tab, b.ctl, n);
  kb_q_cond<<<1, 1, 0, s>>>(h, b.ctl);
  return cudaGetLastError();
}

cudaError_t launch_batch_sweep_cond(const BatchLaunch& b, cudaGraphConditionalHandle h,
                                    cudaStream_t s) {
  kb_q_cond<<<1, 1, 0, s>>>(h, b.ctl);
  return cudaGetLastError();
}

}  // namespace swfd
