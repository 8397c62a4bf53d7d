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
constexpr int UB_BATCH = 8;                    // chunks the resolver stages at a time

// one chunk's summary (terms m0 .. m0 + UB_CHUNK - 1 of one sum)
struct UbChunk {
  double sum, asum;          // terms: FP64 sum and absolute sum (estimates)
  unsigned long long qtot;   // speculate: integer increments of the non-event terms
  int nev;                   // events (> UB_EVC: the chunk is added term by term)
  int pad;
  int ev_pos[UB_EVC];        // position in the chunk
  unsigned long long ev_q[UB_EVC];  // integer prefix of the chunk at the event
  double ev_t[UB_EVC];       // the term
  long long run_lo[UB_EVC + 1], run_hi[UB_EVC + 1];  // run k: least / largest
                             // (prefix since the run's start + floor of the term)
  int run_g[UB_EVC + 1];     // run k: guessed biased exponent | sign << 11 (-2: empty)
  int pad2;
};

__host__ __device__ inline int64_t ub_terms(const Params& p) {
  return p.g.ndim == 1 ? (int64_t)p.g.nx + 6 : (int64_t)p.g.nx * p.g.ny;
}
__host__ __device__ inline int64_t ub_chunks(int64_t n) { return (n + UB_CHUNK - 1) / UB_CHUNK; }

static size_t ub_bytes(int64_t n, int nsum) {
  const size_t t = ((size_t)nsum * n * sizeof(double) + 255) & ~(size_t)255;
  return t + (size_t)nsum * ub_chunks(n) * sizeof(UbChunk) + 256;
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
                                                               UbChunk* __restrict__ ch) {
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
  if (threadIdx.x == 0) {
    ch[c * nch + blockIdx.x].sum = s;
    ch[c * nch + blockIdx.x].asum = a;
  }
}

// the same over a flat array: t(m) = w * x(m) (the test entry point)
__global__ void __launch_bounds__(UB_THREADS) k_ub_terms_flat(const double* __restrict__ x, int64_t n,
                                                              double w, double* __restrict__ T,
                                                              UbChunk* __restrict__ ch) {
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
  if (threadIdx.x == 0) {
    ch[blockIdx.x].sum = s;
    ch[blockIdx.x].asum = a;
  }
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
__global__ void __launch_bounds__(UB_THREADS) k_ub_spec(const double* __restrict__ T, int64_t n,
                                                        UbChunk* __restrict__ ch) {
  const int c = blockIdx.y, tid = threadIdx.x;
  const int64_t nch = ub_chunks(n);
  const double* t_c = T + c * n;
  UbChunk* chc = ch + c * nch;
  UbChunk& C = chc[blockIdx.x];
  __shared__ int s_last[UB_THREADS];
  __shared__ unsigned long long s_evq[UB_EVC];
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
    ps += chc[k].sum;
    pa += chc[k].asum;
  }
  ps = ub_block_sum(ps);
  pa = ub_block_sum(pa);
  // this thread's terms
  const int64_t m0 = (int64_t)blockIdx.x * UB_CHUNK + tid * UB_PER;
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
        C.ev_pos[k] = tid * UB_PER + e;
        C.ev_q[k] = q;
        C.ev_t[k] = t[e];
        s_evq[k] = q;
      }
      ++k;
    } else {
      if (k <= UB_EVC) s_g[k] = gb[e];  // the same for every term of the run
      q += (unsigned long long)(fl[e] + ((upm >> e) & 1u));
    }
  }
  if (tid == 0) {
    C.qtot = qtot;
    C.nev = etot;
  }
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
  for (int r = tid; r <= min(etot, UB_EVC); r += UB_THREADS) {
    C.run_lo[r] = s_lo[r];
    C.run_hi[r] = s_hi[r];
    C.run_g[r] = s_g[r];
  }
}

// ---------------------------------------------------------------------------
// resolve
// ---------------------------------------------------------------------------
// one chunk, in thread 0: terms m0 .. m1-1 of the sum (t_c = its terms).
// Within a run whose first prefix is checked in range, a prefix that leaves
// the range does so by less than 2^54 (no step exceeds 2^53 + 1 units), so
// the recorded least and largest prefixes expose it before any wrap-around.
__device__ double ub_resolve_chunk(const UbChunk& C, const double* __restrict__ t_c, int64_t m0,
                                   int64_t m1, double s) {
  const int nev = C.nev;
  if (nev > UB_EVC) {  // too many events for the summary: term by term
    for (int64_t m = m0; m < m1; ++m) s = s + t_c[m];
    return s;
  }
  unsigned long long qprev = 0;
  int start = 0;
  for (int j = 0; j <= nev; ++j) {
    const unsigned long long qend = j < nev ? C.ev_q[j] : C.qtot;
    const int stop = j < nev ? C.ev_pos[j] : (int)(m1 - m0);
    if (stop > start) {  // the run of terms start .. stop-1
      bool ok = false;
      const unsigned long long sb = (unsigned long long)__double_as_longlong(s);
      const int eb = (int)((sb >> 52) & 0x7ff), neg = (int)(sb >> 63);
      if (eb != 0 && eb != 0x7ff && (eb | (neg << 11)) == C.run_g[j]) {
        const long long M = (long long)((sb & 0xfffffffffffffull) | (1ull << 52));
        if (C.run_lo[j] >= (1ll << 52) - M && C.run_hi[j] <= (1ll << 53) - 1 - M) {
          // every step of the run is its integer step: the sum is M + R in units of u
          const unsigned long long val = (unsigned long long)(M + (long long)(qend - qprev));
          unsigned long long bits = (val == (1ull << 53))
                                        ? ((unsigned long long)(eb + 1) << 52)
                                        : (((unsigned long long)eb << 52) | (val - (1ull << 52)));
          bits |= (unsigned long long)neg << 63;
          s = __longlong_as_double((long long)bits);
          ok = true;
        }
      }
      if (!ok)
        for (int m = start; m < stop; ++m) s = s + t_c[m0 + m];
    }
    if (j < nev) {
      s = s + C.ev_t[j];
      qprev = C.ev_q[j];
      start = C.ev_pos[j] + 1;
    }
  }
  return s;
}

__global__ void __launch_bounds__(UB_THREADS) k_ub_resolve(const double* __restrict__ T, int64_t n,
                                                           const UbChunk* __restrict__ ch,
                                                           double* __restrict__ out) {
  extern __shared__ unsigned long long ub_stage[];
  UbChunk* sb = (UbChunk*)ub_stage;
  const int c = blockIdx.x;
  const int64_t nch = ub_chunks(n);
  const double* t_c = T + c * n;
  const UbChunk* chc = ch + c * nch;
  double s = 0.0;
  constexpr int W = (int)(sizeof(UbChunk) / 8);
  for (int64_t b0 = 0; b0 < nch; b0 += UB_BATCH) {
    const int nb = (int)min((int64_t)UB_BATCH, nch - b0);
    const unsigned long long* src = (const unsigned long long*)(chc + b0);
    for (int w = threadIdx.x; w < nb * W; w += blockDim.x) ub_stage[w] = src[w];
    __syncthreads();
    if (threadIdx.x == 0)
      for (int q = 0; q < nb; ++q) {
        const int64_t m0 = (b0 + q) * UB_CHUNK;
        s = ub_resolve_chunk(sb[q], t_c, m0, min(n, m0 + UB_CHUNK), s);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = s;
}

static cudaError_t ub_finish(const double* T, int64_t n, int nsum, UbChunk* ch, double* out,
                             cudaStream_t s) {
  const dim3 grid((unsigned)ub_chunks(n), nsum);
  k_ub_spec<<<grid, UB_THREADS, 0, s>>>(T, n, ch);
  k_ub_resolve<<<nsum, UB_THREADS, UB_BATCH * sizeof(UbChunk), s>>>(T, n, ch, out);
  return cudaGetLastError();
}

static void ub_carve(void* scratch, int64_t n, int nsum, double** T, UbChunk** ch) {
  *T = (double*)scratch;
  const size_t t = ((size_t)nsum * n * sizeof(double) + 255) & ~(size_t)255;
  *ch = (UbChunk*)((char*)scratch + t);
}

// u_bar of the state into dsc->ubar: three kernels
cudaError_t launch_ubar(const Params& p, const double* u, DevScalars* dsc, void* scratch,
                        cudaStream_t s) {
  const int64_t n = ub_terms(p);
  double* T;
  UbChunk* ch;
  ub_carve(scratch, n, p.g.nc, &T, &ch);
  k_ub_terms_state<<<dim3((unsigned)ub_chunks(n), p.g.nc), UB_THREADS, 0, s>>>(p, u, T, ch);
  return ub_finish(T, n, p.g.nc, ch, dsc->ubar, s);
}

size_t seq_sum_scratch_bytes(int64_t n) { return ub_bytes(n, 1); }

// s = 0; s = s + w*x(m), m = 0..n-1, into *out (device)
cudaError_t launch_seq_sum(const double* x, int64_t n, double w, double* out, void* scratch,
                           cudaStream_t s) {
  if (n <= 0) return cudaMemsetAsync(out, 0, sizeof(double), s);
  double* T;
  UbChunk* ch;
  ub_carve(scratch, n, 1, &T, &ch);
  k_ub_terms_flat<<<(unsigned)ub_chunks(n), UB_THREADS, 0, s>>>(x, n, w, T, ch);
  return ub_finish(T, n, 1, ch, out, s);
}

}  // namespace swfd
