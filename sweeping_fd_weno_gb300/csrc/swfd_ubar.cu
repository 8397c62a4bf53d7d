// swfd_ubar.cu -- u_bar of sweep_lim: the reference's sequential weighted
// sums (2D j-outer/i-inner, ex3_vortex_accuracy_2d/main.f90:913-920; 1D the
// dot_product over -2..n+3, ex2_sedov_1d/main.f90:581-583), rounded step by
// step in the reference's order and evaluated with the whole GPU.
//
// The sum is s(m) = fl(s(m-1) + t(m)).  While s stays inside one binade
// [2^E, 2^(E+1)) with one sign, a step is an integer addition in units of
// u = 2^(E-52) (sum_classify: the rounded quotient t/u, exact); a step that
// leaves the binade, is a rounding tie, meets a zero or subnormal sum or a
// term beyond the binade is one hardware addition -- an event.
//
// Three kernels per sum (one sum per component):
//  terms      t(m) into a contiguous array (all SMs), and the FP64 sum and
//             absolute sum of each chunk of UB_CHUNK terms (estimates);
//  speculate  one block per chunk: an FP64 estimate of the running sum
//             before and after each term (the chunk's start from the FP64
//             chunk sums, then a block scan) gives every term a guessed binade
//             and sign.  A term whose guess is uncertain (within the estimate's
//             error bound of a binade edge or of zero), whose guess changes
//             across its step, or which does not classify under its guess, is
//             an event; every other term is classified under its guess, once.
//             The chunk records its events (position, integer prefix, term)
//             and, for each run of terms between events, its guess and the
//             least and largest integer prefix reached inside it;
//  resolve    one thread per sum walks the chunks, runs and events in order.
//             A run is applied as one integer addition after checking, against
//             the exact running sum, that the sum lies in the run's guessed
//             binade and that every prefix of the run keeps it there -- then
//             each of its steps is the integer step, so the result is exact
//             whatever the guesses were; a run whose check fails is added term
//             by term.  An event is one hardware addition.
// The result is the sequential loop's, bit for bit.  The work per term runs
// once, spread over the GPU; only the walk over runs and events is serial.
#include "swfd_sweep.cuh"

namespace swfd {

constexpr int UB_THREADS = 256;
constexpr int UB_PER = 8;
constexpr int UB_CHUNK = UB_THREADS * UB_PER;  // 2048 terms
constexpr int UB_EVC = 128;                    // events of a chunk on the fast path
constexpr int UB_RCAP = 640;                   // run records the resolver stages at a time
constexpr int UB_ECAP = 640;                   // event records the resolver stages at a time

// one chunk's summary (terms m0 .. m0 + UB_CHUNK - 1 of one sum): its
// estimates, its event count, and UB_EVC + 1 run and UB_EVC event records, of
// which the first nev + 1 and nev are used (runs and events alternate: run 0,
// event 0, run 1, ..., run nev)
struct UbEst {
  double sum, asum;  // terms: FP64 sum and absolute sum of the chunk (estimates)
};
struct UbRun {
  long long lo, hi;          // least / largest (prefix since the run's start + floor)
  unsigned long long rtot;   // sum of the run's integer increments
  int g;                     // guessed biased exponent | sign << 11
  int start, count;          // its terms: chunk positions start .. start + count - 1
  int pad;
};
struct UbEv {
  double t;                  // the term, added in hardware
  long long pad;
};

__host__ __device__ inline int64_t ub_terms(const Params& p) {
  return p.g.ndim == 1 ? (int64_t)p.g.nx + 6 : (int64_t)p.g.nx * p.g.ny;
}
__host__ __device__ inline int64_t ub_chunks(int64_t n) { return (n + UB_CHUNK - 1) / UB_CHUNK; }

struct UbScratch {
  double* T;      // nsum x n terms
  UbEst* est;     // nsum x nch
  int* nev;       // nsum x nch (> UB_EVC: the chunk is added term by term)
  UbRun* runs;    // nsum x nch x (UB_EVC + 1)
  UbEv* evs;      // nsum x nch x UB_EVC
};

static size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }
static size_t ub_bytes(int64_t n, int nsum) {
  const size_t nc = (size_t)nsum * ub_chunks(n);
  return a256(nsum * n * sizeof(double)) + a256(nc * sizeof(UbEst)) + a256(nc * sizeof(int)) +
         a256(nc * (UB_EVC + 1) * sizeof(UbRun)) + a256(nc * UB_EVC * sizeof(UbEv)) + 256;
}
static UbScratch ub_carve(void* scratch, int64_t n, int nsum) {
  const size_t nc = (size_t)nsum * ub_chunks(n);
  char* c = (char*)scratch;
  UbScratch u;
  u.T = (double*)c;
  c += a256(nsum * n * sizeof(double));
  u.est = (UbEst*)c;
  c += a256(nc * sizeof(UbEst));
  u.nev = (int*)c;
  c += a256(nc * sizeof(int));
  u.runs = (UbRun*)c;
  c += a256(nc * (UB_EVC + 1) * sizeof(UbRun));
  u.evs = (UbEv*)c;
  return u;
}
size_t ubar_scratch_bytes(const Params& p) { return ub_bytes(ub_terms(p), p.g.nc); }

// ---------------------------------------------------------------------------
// block helpers (UB_THREADS threads)
// ---------------------------------------------------------------------------
template <class V, class Op>
__device__ __forceinline__ V ub_warp_incl(V v, Op op) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const V o = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v = op(v, o);
  }
  return v;
}

// block exclusive scan of two values; *tota, *totb receive the block totals
template <class A, class B>
__device__ void ub_block_excl(A a, B b, A& ea, B& eb, A* tota, B* totb) {
  __shared__ A sa[UB_THREADS / 32];
  __shared__ B sb[UB_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const A ia = ub_warp_incl(a, [](A x, A y) { return x + y; });
  const B ib = ub_warp_incl(b, [](B x, B y) { return x + y; });
  if (lane == 31) {
    sa[wid] = ia;
    sb[wid] = ib;
  }
  __syncthreads();
  A pa = A(0);
  B pb = B(0);
  for (int k = 0; k < wid; ++k) {
    pa = pa + sa[k];
    pb = pb + sb[k];
  }
  ea = pa + (ia - a);
  eb = pb + (ib - b);
  if (tota) {
    A ta = A(0);
    B tb = B(0);
    for (int k = 0; k < UB_THREADS / 32; ++k) {
      ta = ta + sa[k];
      tb = tb + sb[k];
    }
    *tota = ta;
    *totb = tb;
  }
  __syncthreads();
}

__device__ __forceinline__ double ub_block_sum(double v) {
  __shared__ double red[UB_THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int k = 0; k < UB_THREADS / 32; ++k) t += red[k];
  __syncthreads();
  return t;
}

// ---------------------------------------------------------------------------
// terms
// ---------------------------------------------------------------------------
// u_bar terms of component blockIdx.y: 2D w*u over the interior in j-outer /
// i-inner order with w = 1/(nx*ny); 1D u*w over -2..n+3 with w = 1/(n+6)
__global__ void __launch_bounds__(UB_THREADS) k_ub_terms_state(Params p, const double* __restrict__ u,
                                                               double* __restrict__ T,
                                                               UbEst* __restrict__ est) {
  const Geom& g = p.g;
  const int c = blockIdx.y;
  const int64_t n = ub_terms(p), nch = ub_chunks(n);
  const double* pl = u + c * g.plane;
  const int64_t m0 = (int64_t)blockIdx.x * UB_CHUNK + threadIdx.x * UB_PER;
  double s = 0.0, a = 0.0;
  if (m0 < n) {
    const int k = (int)min((int64_t)UB_PER, n - m0);
    double* out = T + c * n + m0;
    if (g.ndim == 1) {
      const double w = 1 / ((double)g.nx + 6);
      for (int e = 0; e < k; ++e) {
        const double t = pl[m0 + e] * w;
        out[e] = t;
        s += t;
        a += fabs(t);
      }
    } else {
      const double w = 1. / ((double)g.nx * (double)g.ny);
      int i = (int)(m0 % g.nx), j = (int)(m0 / g.nx);
      for (int e = 0; e < k; ++e) {
        const double t = w * pl[g.at(i + 1, j + 1)];
        out[e] = t;
        s += t;
        a += fabs(t);
        if (++i == g.nx) {
          i = 0;
          ++j;
        }
      }
    }
  }
  s = ub_block_sum(s);
  a = ub_block_sum(a);
  if (threadIdx.x == 0) est[c * nch + blockIdx.x] = UbEst{s, a};
}

// the same over a flat array: t(m) = w * x(m) (the test entry point)
__global__ void __launch_bounds__(UB_THREADS) k_ub_terms_flat(const double* __restrict__ x, int64_t n,
                                                              double w, double* __restrict__ T,
                                                              UbEst* __restrict__ est) {
  const int64_t m0 = (int64_t)blockIdx.x * UB_CHUNK + threadIdx.x * UB_PER;
  double s = 0.0, a = 0.0;
  for (int e = 0; e < UB_PER && m0 + e < n; ++e) {
    const double t = w * x[m0 + e];
    T[m0 + e] = t;
    s += t;
    a += fabs(t);
  }
  s = ub_block_sum(s);
  a = ub_block_sum(a);
  if (threadIdx.x == 0) est[blockIdx.x] = UbEst{s, a};
}

// ---------------------------------------------------------------------------
// speculate
// ---------------------------------------------------------------------------
// guessed binade and sign of a running sum from its estimate x, whose error
// is below `margin`: the biased exponent | sign << 11, or -1 when x is within
// margin of a binade edge or of zero, or not a normal binary64
__device__ __forceinline__ int ub_guess(double x, double margin) {
  const unsigned long long xb = (unsigned long long)__double_as_longlong(x);
  const int eb = (int)((xb >> 52) & 0x7ff);
  if (eb == 0 || eb == 0x7ff) return -1;
  const double ax = fabs(x);
  const double lo = __longlong_as_double((long long)((unsigned long long)eb << 52));  // 2^E
  if (!(ax - lo > margin) || !(2.0 * lo - ax > margin)) return -1;
  return eb | (int)((xb >> 63) << 11);
}
// The estimate's error: the sequentially rounded sum of m terms differs from
// the exact one by at most m/2 units of its largest binade, and the estimate
// (chunk sums, a block scan, a thread's additions) from the exact sum by far
// less -- so (m + 64) * 2^-52 of the absolute sum of the terms bounds both.
// The bound only sets which terms are treated as events: the resolver's
// checks keep the result exact whatever the guesses.
__global__ void __launch_bounds__(UB_THREADS) k_ub_spec(UbScratch us, int64_t n) {
  const int c = blockIdx.y, tid = threadIdx.x;
  const int64_t nch = ub_chunks(n), ci = c * nch + blockIdx.x;
  const double* t_c = us.T + c * n;
  const UbEst* estc = us.est + c * nch;
  UbRun* runs = us.runs + ci * (UB_EVC + 1);
  UbEv* evs = us.evs + ci * UB_EVC;
  __shared__ int s_last[UB_THREADS];
  __shared__ unsigned long long s_evq[UB_EVC];
  __shared__ int s_evpos[UB_EVC];
  __shared__ long long s_lo[UB_EVC + 1], s_hi[UB_EVC + 1];
  __shared__ int s_g[UB_EVC + 1];
  for (int k = tid; k <= UB_EVC; k += UB_THREADS) {
    s_lo[k] = LLONG_MAX;
    s_hi[k] = LLONG_MIN;
    s_g[k] = -2;
  }
  // the running sum's estimate at the chunk's start
  double ps = 0.0, pa = 0.0;
  for (int64_t k = tid; k < (int64_t)blockIdx.x; k += UB_THREADS) {
    ps += estc[k].sum;
    pa += estc[k].asum;
  }
  ps = ub_block_sum(ps);
  pa = ub_block_sum(pa);
  // this thread's terms
  const int64_t cm0 = (int64_t)blockIdx.x * UB_CHUNK;
  const int nvalid = (int)min((int64_t)UB_CHUNK, n - cm0);
  const int64_t m0 = cm0 + tid * UB_PER;
  const int kv = m0 < n ? (int)min((int64_t)UB_PER, n - m0) : 0;
  double t[UB_PER];
  double ls = 0.0, la = 0.0;
#pragma unroll
  for (int e = 0; e < UB_PER; ++e) {
    t[e] = e < kv ? t_c[m0 + e] : 0.0;
    ls += t[e];
    la += fabs(t[e]);
  }
  double xs, xa;
  ub_block_excl(ls, la, xs, xa, (double*)nullptr, (double*)nullptr);
  double x = ps + xs;
  const double margin = (pa + xa + la) * 0x1p-52 * (double)(m0 + UB_PER + 64);
  int gb[UB_PER];
#pragma unroll
  for (int e = 0; e < UB_PER; ++e) {
    gb[e] = ub_guess(x, margin);
    x += t[e];
  }
  const int ga_last = kv > 0 ? ub_guess(x, margin) : -3;
  s_last[tid] = ga_last;
  __syncthreads();
  // classify each term under its guess; events
  long long fl[UB_PER];
  unsigned upm = 0, evm = 0;
  unsigned long long rsum = 0;
#pragma unroll
  for (int e = 0; e < UB_PER; ++e) {
    fl[e] = 0;
    if (e >= kv) continue;
    const int ga = (e + 1 < kv) ? gb[e + 1] : ga_last;
    long long r = 0;
    int bad = 1;
    if (gb[e] >= 0) sum_classify(t[e], gb[e] >> 11, gb[e] & 0x7ff, fl[e], r, bad);
    bool ev = bad || gb[e] < 0 || ga < 0 || ga != gb[e];
    // the previous thread's estimate after its last term must agree with
    // this one's before its first (they are rounded apart)
    if (e == 0 && tid > 0 && s_last[tid - 1] != gb[0]) ev = true;
    if (ev) {
      evm |= 1u << e;
    } else {
      upm |= (unsigned)(r - fl[e]) << e;
      rsum += (unsigned long long)r;
    }
  }
  unsigned long long qt, qtot;
  int et, etot;
  ub_block_excl(rsum, __popc(evm), qt, et, &qtot, &etot);
  // events, and each run's guess
  unsigned long long q = qt;
  int k = et;
#pragma unroll
  for (int e = 0; e < UB_PER; ++e) {
    if (e >= kv) continue;
    if ((evm >> e) & 1u) {
      if (k < UB_EVC) {
        evs[k].t = t[e];
        s_evq[k] = q;
        s_evpos[k] = tid * UB_PER + e;
      }
      ++k;
    } else {
      if (k <= UB_EVC) s_g[k] = gb[e];  // the same for every term of the run
      q += (unsigned long long)(fl[e] + ((upm >> e) & 1u));
    }
  }
  if (tid == 0) us.nev[ci] = etot;
  __syncthreads();
  // each run's range of (prefix since its start + floor of the term)
  q = qt;
  k = et;
#pragma unroll
  for (int e = 0; e < UB_PER; ++e) {
    if (e >= kv) continue;
    if ((evm >> e) & 1u) {
      ++k;
    } else {
      if (k <= UB_EVC) {
        const unsigned long long q0 = k ? s_evq[k - 1] : 0ull;
        const long long v = (long long)((q - q0) + (unsigned long long)fl[e]);
        atomicMin(&s_lo[k], v);
        atomicMax(&s_hi[k], v);
      }
      q += (unsigned long long)(fl[e] + ((upm >> e) & 1u));
    }
  }
  __syncthreads();
  if (etot > UB_EVC) return;  // added term by term
  for (int r = tid; r <= etot; r += UB_THREADS) {
    const int start = r ? s_evpos[r - 1] + 1 : 0;
    const int stop = r < etot ? s_evpos[r] : nvalid;
    const unsigned long long qa = r ? s_evq[r - 1] : 0ull, qb = r < etot ? s_evq[r] : qtot;
    runs[r] = UbRun{s_lo[r], s_hi[r], qb - qa, s_g[r], start, stop - start, 0};
  }
}

// ---------------------------------------------------------------------------
// resolve
// ---------------------------------------------------------------------------
// one chunk, in thread 0: terms m0 .. m0+nvalid-1 of the sum (t_c its terms),
// nev events, its runs and events staged in shared memory.  Within a run
// whose start is checked in range, a prefix that leaves the range does so by
// less than 2^54 (no step exceeds 2^53 + 1 units), so the recorded least and
// largest prefixes expose it before any wrap-around.
__device__ double ub_resolve_chunk(int nev, const UbRun* runs, const UbEv* evs,
                                   const double* __restrict__ t_c, int64_t m0, int nvalid,
                                   double s) {
  if (nev > UB_EVC) {  // too many events for the summary: term by term
    for (int m = 0; m < nvalid; ++m) s = s + t_c[m0 + m];
    return s;
  }
  for (int j = 0; j <= nev; ++j) {
    const UbRun& R = runs[j];
    if (R.count > 0) {
      bool ok = false;
      const unsigned long long sb = (unsigned long long)__double_as_longlong(s);
      const int eb = (int)((sb >> 52) & 0x7ff), neg = (int)(sb >> 63);
      if (eb != 0 && eb != 0x7ff && (eb | (neg << 11)) == R.g) {
        const long long M = (long long)((sb & 0xfffffffffffffull) | (1ull << 52));
        if (R.lo >= (1ll << 52) - M && R.hi <= (1ll << 53) - 1 - M) {
          // every step of the run is its integer step: the sum is M + R in units of u
          const unsigned long long val = (unsigned long long)(M + (long long)R.rtot);
          unsigned long long bits = (val == (1ull << 53))
                                        ? ((unsigned long long)(eb + 1) << 52)
                                        : (((unsigned long long)eb << 52) | (val - (1ull << 52)));
          bits |= (unsigned long long)neg << 63;
          s = __longlong_as_double((long long)bits);
          ok = true;
        }
      }
      if (!ok)
        for (int m = R.start; m < R.start + R.count; ++m) s = s + t_c[m0 + m];
    }
    if (j < nev) s = s + evs[j].t;
  }
  return s;
}

// one block per sum: batches of up to UB_THREADS chunks whose used records fit
// the staging arrays are copied to shared memory by all threads, then walked
// by thread 0
__global__ void __launch_bounds__(UB_THREADS) k_ub_resolve(UbScratch us, int64_t n,
                                                           double* __restrict__ out) {
  __shared__ UbRun s_runs[UB_RCAP];
  __shared__ UbEv s_evs[UB_ECAP];
  __shared__ int s_nev[UB_THREADS], s_ro[UB_THREADS], s_eo[UB_THREADS];
  const int c = blockIdx.x, tid = threadIdx.x;
  const int64_t nch = ub_chunks(n);
  const double* t_c = us.T + c * n;
  double s = 0.0;
  for (int64_t b0 = 0; b0 < nch;) {
    const int64_t k = b0 + tid;
    const int nev = k < nch ? us.nev[c * nch + k] : 0;
    const int rc = (k < nch && nev <= UB_EVC) ? nev + 1 : 0;
    const int ec = (k < nch && nev <= UB_EVC) ? nev : 0;
    int ro, eo;
    ub_block_excl(rc, ec, ro, eo, (int*)nullptr, (int*)nullptr);
    // the chunks that fit form a prefix of the batch (the offsets only grow)
    const bool fits = k < nch && ro + rc <= UB_RCAP && eo + ec <= UB_ECAP;
    const int nb = __syncthreads_count(fits);
    s_nev[tid] = nev;
    s_ro[tid] = ro;
    s_eo[tid] = eo;
    if (fits) {
      const UbRun* rs = us.runs + (c * nch + k) * (UB_EVC + 1);
      const UbEv* es = us.evs + (c * nch + k) * UB_EVC;
      for (int r = 0; r < rc; ++r) s_runs[ro + r] = rs[r];
      for (int e = 0; e < ec; ++e) s_evs[eo + e] = es[e];
    }
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < nb; ++q) {
        const int64_t m0 = (b0 + q) * UB_CHUNK;
        s = ub_resolve_chunk(s_nev[q], s_runs + s_ro[q], s_evs + s_eo[q], t_c, m0,
                             (int)min((int64_t)UB_CHUNK, n - m0), s);
      }
    __syncthreads();
    b0 += nb;
  }
  if (tid == 0) out[c] = s;
}

static cudaError_t ub_finish(const UbScratch& us, int64_t n, int nsum, double* out,
                             cudaStream_t s) {
  const dim3 grid((unsigned)ub_chunks(n), nsum);
  k_ub_spec<<<grid, UB_THREADS, 0, s>>>(us, n);
  k_ub_resolve<<<nsum, UB_THREADS, 0, s>>>(us, n, out);
  return cudaGetLastError();
}

// u_bar of the state into dsc->ubar: three kernels
cudaError_t launch_ubar(const Params& p, const double* u, DevScalars* dsc, void* scratch,
                        cudaStream_t s) {
  const int64_t n = ub_terms(p);
  const UbScratch us = ub_carve(scratch, n, p.g.nc);
  k_ub_terms_state<<<dim3((unsigned)ub_chunks(n), p.g.nc), UB_THREADS, 0, s>>>(p, u, us.T, us.est);
  return ub_finish(us, n, p.g.nc, dsc->ubar, s);
}

size_t seq_sum_scratch_bytes(int64_t n) { return ub_bytes(n, 1); }

// s = 0; s = s + w*x(m), m = 0..n-1, into *out (device)
cudaError_t launch_seq_sum(const double* x, int64_t n, double w, double* out, void* scratch,
                           cudaStream_t s) {
  if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(double), s);
  const UbScratch us = ub_carve(scratch, n, 1);
  k_ub_terms_flat<<<(unsigned)ub_chunks(n), UB_THREADS, 0, s>>>(x, n, w, us.T, us.est);
  return ub_finish(us, n, 1, out, s);
}

}  // namespace swfd
