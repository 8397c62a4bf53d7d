// swfd_sweep.cuh -- device functions of the sweeping post-process, shared by
// the single-instance kernels (swfd_sweep.cu) and the batched ones
// (swfd_batch.cu).
#pragma once

#include "swfd_device.cuh"

namespace swfd {

// position -> cell offset; ordering 1 = I (column by column), 2 = II (row by
// row), 0 = 1D index order over -2..n+3
__device__ __forceinline__ int64_t pos_cell(const Geom& g, int ordering, int64_t pos) {
  if (ordering == 0) return pos;  // 1D: position p is cell p-2, offset p
  int i, j;
  if (ordering == 1) {
    j = ((int)pos / g.nx) + 1;
    int t = ((int)pos % g.nx);
    i = (j & 1) ? t + 1 : g.nx - t;
  } else {
    i = ((int)pos / g.ny) + 1;
    int t = ((int)pos % g.ny);
    j = (i & 1) ? t + 1 : g.ny - t;
  }
  return g.at(i, j);
}

__host__ __device__ __forceinline__ int64_t npos(const Geom& g) {
  return g.ndim == 1 ? (int64_t)g.LI : (int64_t)g.nx * g.ny;
}

// pressure as the sweep computes it
// (2D ex3_vortex_accuracy_2d/main.f90:946, 1D ex2_sedov_1d/main.f90:603).
// The divisions are sd::div and the products by 0.5 exponent shifts (the
// same bits as the IEEE operations): a sweep pass is a chain of dependent
// nodal adjustments, and GB300's FP64 pipe has a long latency, so the
// integer-pipe division shortens every step of that chain.
__device__ __forceinline__ double sweep_pres(const Geom& g, double g1, const double* v) {
  if (g.ndim == 1) return g1 * (v[2] - tdiv(tscale<-1>(v[1] * v[1]), v[0]));
  return g1 * (v[3] - tdiv(tscale<-1>(v[1] * v[1] + v[2] * v[2]), v[0]));
}

// nod_lim (ex3_vortex_accuracy_2d/main.f90:846-884; 1D ex2_sedov_1d/main.f90:517-560)
__device__ inline void nod_lim(const Geom& g, double g1, double eps, const double* v1, const double* v2,
                        const double* vb, double* out, long long& npos_, long long& nneg) {
  double t;
  if (g.ndim == 1) {
    double p1 = g1 * (v1[2] - tscale<-1>(tdiv(v1[1] * v1[1], v1[0])));
    double p2 = g1 * (v2[2] - tscale<-1>(tdiv(v2[1] * v2[1], v2[0])));
    if (p2 > eps) {
      t = tdiv(p1 - eps, p1 - p2);
      ++npos_;
    } else {
      double pb = g1 * (vb[2] - tscale<-1>(tdiv(vb[1] * vb[1], vb[0])));
      double t_1 = tdiv(p1 - eps, p1 - pb);
      double d12 = sqrt(dsq(v2[2] - v1[2]) + dsq(v2[1] - v1[1]) + dsq(v2[0] - v1[0]));
      double d1b = sqrt(dsq(vb[2] - v1[2]) + dsq(vb[1] - v1[1]) + dsq(vb[0] - v1[0]));
      t = fmin(tdiv(t_1 * d1b, d12), 0.25);
      ++nneg;
    }
  } else {
    double p1 = g1 * (v1[3] - tdiv(tscale<-1>(v1[1] * v1[1] + v1[2] * v1[2]), v1[0]));
    double p2 = g1 * (v2[3] - tdiv(tscale<-1>(v2[1] * v2[1] + v2[2] * v2[2]), v2[0]));
    if (p2 > eps) {
      t = tdiv(p1 - eps, p1 - p2);
      ++npos_;
    } else {
      double pb = g1 * (vb[3] - tdiv(tscale<-1>(vb[1] * vb[1] + vb[2] * vb[2]), vb[0]));
      double t_1 = tdiv(p1 - eps, p1 - pb);
      double d12 = sqrt(dsq(v2[3] - v1[3]) + dsq(v2[2] - v1[2]) + dsq(v2[1] - v1[1]) +
                        dsq(v2[0] - v1[0]));
      double d1b = sqrt(dsq(vb[3] - v1[3]) + dsq(vb[2] - v1[2]) + dsq(vb[1] - v1[1]) +
                        dsq(vb[0] - v1[0]));
      t = fmin(tdiv(t_1 * d1b, d12), 0.25);
      ++nneg;
    }
  }
  for (int c = 0; c < g.nc; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
}


__device__ __forceinline__ unsigned long long order_key(double v) {
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}


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
                                       long long& npos_, long long& nneg, int* fail = nullptr) {
    if (KIND == 1) {
      const double delta = p.g.ndim == 1 ? 1e-13 : 1e-12;
      nx.s[0] = nx.s[0] + 1.0 * (s[0] - delta);
      s[0] = delta;
    } else {
      double vit[4], pi = 0., pp = 0.;
      if (fail) {
        pi = sweep_pres(p.g, p.gamma1, s);
        pp = sweep_pres(p.g, p.gamma1, nx.s);
      }
      nod_lim(p.g, p.gamma1, p.eps, s, nx.s, ub, vit, npos_, nneg);
      for (int c = 0; c < p.g.nc; ++c) {
        double d = s[c] - vit[c];
        s[c] = vit[c];
        nx.s[c] = nx.s[c] + 1.0 * (d);
      }
      // ex6: the pair's total pressure must not increase
      // (ex6_shock_diffraction/main.f90:1413-1423)
      if (fail && pi + pp > sweep_pres(p.g, p.gamma1, s) + sweep_pres(p.g, p.gamma1, nx.s) + p.eps)
        *fail = 1;
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
__device__ inline int64_t run_chain(const Params& p, double* u, int ordering, int forward, int64_t N,
                             int64_t q0, int64_t stop, const double* ub, int* merged,
                             long long& npos_, long long& nneg, int* fail = nullptr) {
  const Geom& g = p.g;
  // the ex6 check runs in the ordering-I passes (ex6_shock_diffraction/main.f90:1413-1423,
  // 1472-1482; the ordering-II checks do not stop)
  int* chk = (KIND == 0 && WRITE && p.sweep_check && ordering == 1) ? fail : nullptr;
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
    cur.step(p, nxt, ub, npos_, nneg, chk);
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


inline size_t sweep_scratch_bytes_impl(const Params& p) {
  const int64_t N = npos(p.g);
  const int64_t W = (N + 31) / 32 + 1;
  return W * 4 + N * 4 * 2 + N * 2 + 64 + 256;
}

__host__ __device__ inline SweepScratch carve(void* base, const Params& p) {
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


// p / u = ip + rem / 2^d relative to the binade with biased exponent eb of a
// running sum of sign neg_s (mirrored to a positive sum): floor (fl) and
// rounded value (r) in units of u; bad = 1 for a tie, an exponent above the
// binade's or a non-finite p
__device__ __forceinline__ void sum_classify(double p, int neg_s, int eb, long long& fl,
                                             long long& r, int& bad) {
  const unsigned long long pb = (unsigned long long)__double_as_longlong(p);
  const int ps = (int)(pb >> 63) ^ neg_s;
  int pe = (int)((pb >> 52) & 0x7ff);
  unsigned long long mp = pb & 0xfffffffffffffull;
  fl = 0;
  r = 0;
  bad = 0;
  if (pe == 0x7ff) {
    bad = 1;
    return;
  }
  if (pe) mp |= 1ull << 52;
  else pe = 1;
  if (mp == 0) return;  // +-0
  const int d = eb - pe;
  if (d < 0) {  // |p / u| >= 2^53: the sum leaves the binade
    bad = 1;
    return;
  }
  unsigned long long ip, rem, half;
  if (d == 0) {
    ip = mp;
    rem = 0;
    half = 1;
  } else if (d < 64) {
    ip = mp >> d;
    rem = mp & ((1ull << d) - 1);
    half = 1ull << (d - 1);
    if (rem == half) {
      bad = 1;
      return;
    }
  } else {  // 0 < |p / u| < 2^-10
    ip = 0;
    rem = 1;
    half = 2;
  }
  const long long up = rem > half ? 1 : 0;
  if (!ps) {
    fl = (long long)ip;
    r = (long long)ip + up;
  } else {
    fl = -(long long)ip - (rem != 0 ? 1 : 0);
    r = -((long long)ip + up);
  }
}

// Cluster-parallel passes (single-instance path).  A cluster is a maximal
// run of flagged positions F[k0..k1] whose dry runs each reach the next
// flagged position (dry_merge[k0..k1-1] = 1, dry_merge[k1] = 0).  One thread
// walks each cluster in order with writes -- exactly the sequential walk
// restricted to the cluster's positions -- and stops if its walk reaches the
// first position of the next cluster, which another thread owns.  The cluster
// saves the original value of every position it walks over (backup), so that
// such a spill can be undone: one warp then restores the later clusters and
// finishes the pass sequentially from the spill.
struct ClusterScratch {
  double* orig;      // per k: nc values of cell(F[k]) when the pass starts
  double* carry;     // per cluster start k: the carried cell state at its stop
  double* backup;    // per position: nc original values of the positions walked
  long long* cnt;    // per cluster start k: positive-neighbour and negative-pair counts
  int* end;          // per cluster start k: last position written
  int* next;         // per cluster start k: index of the next cluster's start (m: none)
  uint8_t* flag;     // per k: 0 not a cluster start, 1 done, 2 stopped at the next
                     // cluster's start, 4 (or'ed) ex6 pressure check failed
};

inline size_t cluster_scratch_bytes(const Params& p) {
  const int64_t N = npos(p.g);
  return (size_t)N * (8 * 4 * 3 + 8 * 2 + 4 * 2 + 1) + 256;
}

__host__ __device__ inline ClusterScratch carve_cluster(void* base, const Params& p) {
  const int64_t N = npos(p.g);
  char* c = (char*)base;
  ClusterScratch s;
  s.orig = (double*)c;
  c += N * 4 * 8;
  s.carry = (double*)c;
  c += N * 4 * 8;
  s.backup = (double*)c;
  c += N * 4 * 8;
  s.cnt = (long long*)c;
  c += N * 2 * 8;
  s.end = (int*)c;
  c += N * 4;
  s.next = (int*)c;
  c += N * 4;
  s.flag = (uint8_t*)c;
  return s;
}

}  // namespace swfd
