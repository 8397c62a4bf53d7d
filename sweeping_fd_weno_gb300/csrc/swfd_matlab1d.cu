// swfd_matlab1d.cu -- the MATLAB script of the reference's first example
// (ex1_double_rarefaction_1d/FD_WENO_Application.m with get_variables.m,
// get_pressure_data.m, scalar_pos.m, apply_sweep.m, swp_alg_triag_nxt.m and
// node_adj_scale_lim_triag.m): SSP-RK3 of a characteristic-wise WENO5 scheme
// with a Lax-Friedrichs alpha per characteristic field, and the sweeps after
// every stage.
//
// The grids are small (the script's problems run 20..801 cells) and a step is
// a chain of short dependent phases, so one thread block runs whole steps:
// the cell- and interface-parallel phases are spread over its threads and
// separated by block barriers; the sweeps flag each pass's bad positions over
// the block and walk the chains from them in thread 0, which also forms the
// weighted means (left-to-right sums).  A
// launch advances up to max_steps steps (the time loop `while t < tFinal`,
// :212, is tested on the device).
//
// Operation order follows the script as MATLAB evaluates it (left to right,
// unary minus before * and /), with x.^2 as x*x, the weighted means as
// left-to-right sums and 3x3 matrix products row by row, left to right.
#include "swfd_internal.h"

namespace swfd {

namespace {

constexpr int MT = 256;  // threads of the block

__device__ __forceinline__ double sqd(double a) { return a * a; }

// scalarWeno (FD_WENO_Application.m:588-629) of the 6 values s[0..5]:
// umOut (value at the right face of s[2] from the left) and upOut (value at
// the same face from the right)
__device__ void scalar_weno(const double* s, double& um_out, double& up_out) {
  const double umm = s[0], um = s[1], u = s[2], up = s[3], upp = s[4], uppp = s[5];
  const double c13 = 1. / 3., c76 = 7. / 6., c116 = 11. / 6., c16 = 1. / 6., c56 = 5. / 6.;
  const double c1312 = 13. / 12., c14 = 1. / 4., eps = 10e-6;
  const double cw1 = 1. / 10., cw2 = 3. / 5., cw3 = 3. / 10.;
  double um1 = c13 * umm - c76 * um + c116 * u;
  double um2 = -c16 * um + c56 * u + c13 * up;
  double um3 = c13 * u + c56 * up - c16 * upp;
  double b1 = c1312 * sqd(umm - 2 * um + u) + c14 * sqd(umm - 4 * um + 3 * u);
  double b2 = c1312 * sqd(um - 2 * u + up) + c14 * sqd(um - up);
  double b3 = c1312 * sqd(u - 2 * up + upp) + c14 * sqd(3 * u - 4 * up + upp);
  double w1 = cw1 / sqd(b1 + eps), w2 = cw2 / sqd(b2 + eps), w3 = cw3 / sqd(b3 + eps);
  double sw = w1 + w2 + w3;
  um_out = w1 / sw * um1 + w2 / sw * um2 + w3 / sw * um3;
  double up1 = c116 * up - c76 * upp + c13 * uppp;
  double up2 = c13 * u + c56 * up - c16 * upp;
  double up3 = -c16 * um + c56 * u + c13 * up;
  b1 = c1312 * sqd(uppp - 2 * upp + up) + c14 * sqd(uppp - 4 * upp + 3 * up);
  b2 = c1312 * sqd(upp - 2 * up + u) + c14 * sqd(upp - u);
  b3 = c1312 * sqd(up - 2 * u + um) + c14 * sqd(3 * up - 4 * u + um);
  w1 = cw1 / sqd(b1 + eps), w2 = cw2 / sqd(b2 + eps), w3 = cw3 / sqd(b3 + eps);
  sw = w1 + w2 + w3;
  up_out = w1 / sw * up1 + w2 / sw * up2 + w3 / sw * up3;
}

// max over the block of three values per thread; NaN-started and fmax-folded
// like MATLAB's max, which skips NaN
__device__ void block_max3(double (&v)[3], double* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    for (int o = 16; o > 0; o >>= 1) v[r] = fmax(v[r], __shfl_xor_sync(0xffffffffu, v[r], o));
    if (lane == 0) sh[r * 8 + w] = v[r];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int r = 0; r < 3; ++r) {
      double m = sh[r * 8];
      for (int k = 1; k < MT / 32; ++k) m = fmax(m, sh[r * 8 + k]);
      sh[24 + r] = m;
    }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < 3; ++r) v[r] = sh[24 + r];
  __syncthreads();
}

// workspace of one solve, carved from `wk` (matlab1d_workspace doubles)
struct Work {
  double *uh;                       // the stage state, 3 x n (component-major)
  double *fP, *fM0;                 // fluxes at faces 1..n (3 x n), left face of cell 1
  double *ro, *m, *E, *v, *p, *sr, *H1;  // padded, index J = 1..n+6
  double *vxm, *hxm, *qm, *cm, *t2;      // Roe averages at J+1/2
};

__device__ Work carve(double* wk, int n) {
  const int L = n + 8;
  Work w;
  w.uh = wk;
  w.fP = wk + 3 * n;
  w.fM0 = wk + 6 * n;
  double* a = wk + 6 * n + 4;
  w.ro = a, w.m = a + L, w.E = a + 2 * L, w.v = a + 3 * L, w.p = a + 4 * L, w.sr = a + 5 * L;
  w.H1 = a + 6 * L, w.vxm = a + 7 * L, w.hxm = a + 8 * L, w.qm = a + 9 * L, w.cm = a + 10 * L;
  w.t2 = a + 11 * L;
  return w;
}

struct Ctx {
  int n, per;
  double g1;
};

// interior cell feeding padded index J (FD_WENO_Step's padding, :394-411)
__device__ __forceinline__ int pad_src(const Ctx& c, int J) {
  if (J <= 3) return c.per ? c.n - 3 + J : 1;
  if (J > c.n + 3) return c.per ? J - c.n - 3 : c.n;
  return J - 3;
}

// FD_WENO_Step (:392-585) on the stage state `in` (component c of interior
// cell i at in[c * ld + i - 1 + off]); fluxes into w.fP / w.fM0
__device__ void fluxes(const Ctx& c, const double* in, int ld, int off, const Work& w,
                       double* sh) {
  const int n = c.n, N = n + 6;
  const double g1 = c.g1;
  for (int J = 1 + threadIdx.x; J <= N; J += MT) {
    const int i = pad_src(c, J) - 1 + off;
    const double r = in[i], mm = in[ld + i], e = in[2 * ld + i];
    w.ro[J] = r, w.m[J] = mm, w.E[J] = e;
    w.v[J] = mm / r;
    w.p[J] = g1 * (e - 1. / 2. * (mm * mm) / r);
  }
  __syncthreads();
  for (int J = 1 + threadIdx.x; J <= N; J += MT) {
    w.sr[J] = sqrt(w.ro[J]);
    w.H1[J] = (w.p[J] + w.E[J]) / w.ro[J];
  }
  __syncthreads();
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  double al[3] = {qnan, qnan, qnan};
  for (int J = 1 + threadIdx.x; J <= N; J += MT) {
    const int Jn = J == N ? 1 : J + 1;
    const double t0 = w.sr[J] / (w.sr[J] + w.sr[Jn]);
    const double t1 = 1 - t0;
    const double vxm = t0 * w.v[J] + t1 * w.v[Jn];
    const double hxm = t0 * w.H1[J] + t1 * w.H1[Jn];
    const double qm = 0.5 * (vxm * vxm);
    const double cm = sqrt(g1 * (hxm - qm));
    w.vxm[J] = vxm, w.hxm[J] = hxm, w.qm[J] = qm, w.cm[J] = cm, w.t2[J] = vxm * cm;
    al[0] = fmax(al[0], fabs(vxm - cm));
    al[1] = fmax(al[1], fabs(vxm));
    al[2] = fmax(al[2], fabs(vxm + cm));
  }
  block_max3(al, sh);
  // the flux at face J+1/2 from cells J-2..J+3 (:445-517); face kk = 0 is
  // the left face of cell 1 (non-periodic: :545-583)
  for (int kk = threadIdx.x; kk <= n; kk += MT) {
    if (kk == 0 && c.per) continue;
    const int J = kk + 3;
    const double V = w.vxm[J], H = w.hxm[J], q = w.qm[J], cc = w.cm[J], T2 = w.t2[J];
    const double rcm = 1 / cc;
    const double b1 = g1 * (rcm * rcm), b2 = q * b1, t0h = V * rcm, t1h = b1 * V, t2h = 0.5 * b1;
    const double Lm[3][3] = {{0.5 * (b2 + t0h), -0.5 * (t1h + rcm), t2h},
                             {1 - b2, t1h, -b1},
                             {0.5 * (b2 - t0h), -0.5 * (t1h - rcm), t2h}};
    double gp[3][6], gm[3][6];
#pragma unroll
    for (int idx = 0; idx < 6; ++idx) {
      const int i = J - 2 + idx;
      const double ro = w.ro[i], mm = w.m[i], e = w.E[i], vv = w.v[i], pp = w.p[i];
      const double uu[3] = {ro, mm, e};
      const double fu[3] = {mm, ro * (vv * vv) + pp, vv * (e + pp)};
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const double ww = Lm[r][0] * uu[0] + Lm[r][1] * uu[1] + Lm[r][2] * uu[2];
        const double gg = Lm[r][0] * fu[0] + Lm[r][1] * fu[1] + Lm[r][2] * fu[2];
        gp[r][idx] = 1. / 2. * (gg + al[r] * ww);
        gm[r][idx] = 1. / 2. * (gg - al[r] * ww);
      }
    }
    double gh[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double um_p, up_p, um_m, up_m;
      scalar_weno(gm[r], um_m, up_m);
      scalar_weno(gp[r], um_p, up_p);
      gh[r] = up_m + um_p;
    }
    const double f0 = 1 * gh[0] + 1 * gh[1] + 1 * gh[2];
    const double f1 = (V - cc) * gh[0] + V * gh[1] + (V + cc) * gh[2];
    const double f2 = (H - T2) * gh[0] + q * gh[1] + (H + T2) * gh[2];
    double* dst = kk >= 1 ? w.fP + (kk - 1) : w.fM0;
    const int ldf = kk >= 1 ? n : 1;
    dst[0] = f0, dst[ldf] = f1, dst[2 * ldf] = f2;
  }
  __syncthreads();
}

// --- the sweeps, sequential in thread 0 (uh is component-major, 3 x n) ---
__device__ __forceinline__ double P14(const double* x) {  // the sweep files' gamma = 1.4
  return (1.4 - 1) * (x[2] - 1. / 2. * ((x[1] * x[1]) / x[0]));
}

// shared memory of the block-cooperative sweep: the flagged positions of a
// pass (n - 1 <= SW_CAP; larger grids take the thread-0 sweep)
constexpr int SW_CAP = 4096;
struct SweepShared {
  int list[SW_CAP];
  int cnt;
  int wcnt[MT / 32];
  double red[MT / 32];
  double red_out, pu;
  double ub[3];
};

struct Sweep {
  double* uh;
  int n;
  double w;  // every weight: ones(1,nSteps)*1/nSteps
  DevScalars* d;
  __device__ void get(int i, double* x) const {
    x[0] = uh[i - 1], x[1] = uh[n + i - 1], x[2] = uh[2 * n + i - 1];
  }
  __device__ void put(int i, const double* x) {
    uh[i - 1] = x[0], uh[n + i - 1] = x[1], uh[2 * n + i - 1] = x[2];
  }
  // get_pressure_data.m
  __device__ void pressure_data(double& pmin, double& pu) const {
    double ra = 0, ma = 0, ea = 0, mn = 0;
    for (int i = 1; i <= n; ++i) {
      double x[3];
      get(i, x);
      const double P = x[2] - 1. / 2. * ((x[1] * x[1]) / x[0]);
      mn = (i == 1) ? P : fmin(mn, P);
      ra = ra + x[0] * w, ma = ma + x[1] * w, ea = ea + x[2] * w;
    }
    pmin = mn;
    pu = ea - 1. / 2. * ((ma * ma) / ra);
  }
  __device__ double rho_min() const {
    double r = 0;
    for (int i = 1; i <= n; ++i) r = (i == 1) ? uh[i - 1] : fmin(r, uh[i - 1]);
    return r;
  }
  // scalar_pos.m
  __device__ void scalar_pos() {
    const double m = 1e-16;
    for (int j = 1; j <= n - 1; ++j) {
      const double vj = uh[j - 1], vp = uh[j];
      if (vj < m) {
        uh[j] = vp + (w / w) * (vj - m);
        uh[j - 1] = m;
      }
    }
    for (int j = n; j >= 2; --j) {
      const double vj = uh[j - 1], vp = uh[j - 2];
      if (vj < m) {
        uh[j - 2] = vp + (w / w) * (vj - m);
        uh[j - 1] = m;
      }
    }
    d->den_count++;
  }
  // node_adj_scale_lim_triag.m
  __device__ void node_adj(const double* v1, const double* v2, const double* vb, double* out) {
    const double epsi = 1e-13;
    double t;
    if (P14(v2) > epsi) {
      t = (P14(v1) - epsi) / (P14(v1) - P14(v2));
      d->t_pos++;
    } else {
      const double t1 = (P14(v1) - epsi) / (P14(v1) - P14(vb));
      const double d1 = sqrt(sqd(vb[2] - v1[2]) + sqd(vb[1] - v1[1]) + sqd(vb[0] - v1[0]));
      const double d2 = sqrt(sqd(v2[2] - v1[2]) + sqd(v2[1] - v1[1]) + sqd(v2[0] - v1[0]));
      t = fmin(t1 * d1 / d2, 0.25);
      d->t_neg++;
    }
    for (int c = 0; c < 3; ++c) out[c] = (1 - t) * v1[c] + t * v2[c];
  }
  // swp_alg_triag_nxt.m, bounded by swp_num
  __device__ void swp_alg(int swp_num) {
    const double epsi = 1e-12;
    double ub[3] = {0, 0, 0};
    for (int c = 0; c < 3; ++c)
      for (int i = 1; i <= n; ++i) ub[c] = ub[c] + uh[c * n + i - 1] * w;
    d->sweep_count++;
    const long long k = d->sweep_count - 1;
    const bool rec = k < d->track_cap;
    d->t_pos = d->t_neg = 0;
    int q;
    for (q = 1; q <= swp_num; ++q) {
      for (int pass = 0; pass < 2; ++pass)
        for (int s = 1; s <= n - 1; ++s) {
          const int j = pass == 0 ? s : n - s + 1, jp = pass == 0 ? j + 1 : j - 1;
          double vj[3], vp[3];
          get(j, vj);
          if (P14(vj) <= epsi || vj[0] < 0) {
            get(jp, vp);
            double vjt[3], nv[3];
            node_adj(vj, vp, ub, vjt);
            for (int c = 0; c < 3; ++c) nv[c] = vp[c] + (w / w) * (vj[c] - vjt[c]);
            put(j, vjt);
            put(jp, nv);
          }
        }
      d->pre_count++;
      double pmin, pu;
      pressure_data(pmin, pu);
      if (pmin > epsi && rho_min() > epsi) break;
    }
    if (q > swp_num) {
      q = swp_num;
      d->fail_count++;
    }
    if (rec) {
      d->tracks[k] = q;
      d->tracks[d->track_cap + k] = (int)d->t_neg;
      d->tracks[2 * d->track_cap + k] = (int)d->t_pos;
    }
  }
  // ---- block-cooperative forms (every thread of the block calls them): the
  // minima and the pass-start flags over the block's threads, the
  // sequential parts (the weighted sums, the adjustments) in thread 0; the
  // same values and counts as the thread-0 forms above ----
  // fmin over the block (NaN is fmin's identity, as in the thread-0 fold)
  __device__ double block_min(double v, SweepShared& S) const {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) S.red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = S.red[0];
      for (int k = 1; k < MT / 32; ++k) m = fmin(m, S.red[k]);
      S.red_out = m;
    }
    __syncthreads();
    const double r = S.red_out;
    __syncthreads();
    return r;
  }
  __device__ double rho_min_par(SweepShared& S) const {
    double v = __longlong_as_double(0x7ff8000000000000ll);
    for (int i = 1 + threadIdx.x; i <= n; i += MT) v = fmin(v, uh[i - 1]);
    return block_min(v, S);
  }
  __device__ void pressure_data_par(double& pmin, double& pu, SweepShared& S) const {
    double v = __longlong_as_double(0x7ff8000000000000ll);
    for (int i = 1 + threadIdx.x; i <= n; i += MT) {
      double x[3];
      get(i, x);
      v = fmin(v, x[2] - 1. / 2. * ((x[1] * x[1]) / x[0]));
    }
    if (threadIdx.x == 0) {  // the weighted means, left to right
      double ra = 0, ma = 0, ea = 0;
      for (int i = 1; i <= n; ++i) {
        double x[3];
        get(i, x);
        ra = ra + x[0] * w, ma = ma + x[1] * w, ea = ea + x[2] * w;
      }
      S.pu = ea - 1. / 2. * ((ma * ma) / ra);
    }
    pmin = block_min(v, S);  // its barriers publish S.pu
    pu = S.pu;
  }
  __device__ static bool sweep_bad(const double* v) { return P14(v) <= 1e-12 || v[0] < 0; }
  // the positions s = 1..n-1 of pass `pass` whose cell is bad on the
  // pass-start state, in pass order, into S.list[0..S.cnt)
  __device__ void flag_list(int pass, SweepShared& S) const {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) S.cnt = 0;
    __syncthreads();
    for (int base = 1; base <= n - 1; base += MT) {
      const int s = base + threadIdx.x;
      bool f = false;
      if (s <= n - 1) {
        double v[3];
        get(pass == 0 ? s : n - s + 1, v);
        f = sweep_bad(v);
      }
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (lane == 0) S.wcnt[wid] = __popc(m);
      __syncthreads();
      int off = S.cnt;
      for (int k = 0; k < wid; ++k) off += S.wcnt[k];
      if (f) S.list[off + __popc(m & ((1u << lane) - 1u))] = s;
      __syncthreads();
      if (threadIdx.x == 0)
        for (int k = 0; k < MT / 32; ++k) S.cnt += S.wcnt[k];
      __syncthreads();
    }
  }
  // one pass from its flagged positions: at a flagged position the cell is
  // unchanged since the pass start, so it adjusts; each adjustment changes the
  // next position's cell, which is checked afresh (the chain goes on while it
  // is bad); a position a chain passed is not visited again -- the visits and
  // adjustments of the sequential pass
  __device__ void walk(int pass, const double* ub, const SweepShared& S) {
    int s_next = 1;
    for (int k = 0; k < S.cnt; ++k) {
      int s = S.list[k];
      if (s < s_next) continue;
      for (;;) {
        const int j = pass == 0 ? s : n - s + 1, jp = pass == 0 ? j + 1 : j - 1;
        double vj[3], vp[3], vjt[3], nv[3];
        get(j, vj);
        get(jp, vp);
        node_adj(vj, vp, ub, vjt);
        for (int c = 0; c < 3; ++c) nv[c] = vp[c] + (w / w) * (vj[c] - vjt[c]);
        put(j, vjt);
        put(jp, nv);
        if (++s > n - 1) break;
        double v2[3];
        get(pass == 0 ? s : n - s + 1, v2);
        if (!sweep_bad(v2)) break;
      }
      s_next = s + 1;
    }
  }
  __device__ void swp_alg_par(int swp_num, SweepShared& S) {
    const double epsi = 1e-12;
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c) {
        double ub = 0;
        for (int i = 1; i <= n; ++i) ub = ub + uh[c * n + i - 1] * w;
        S.ub[c] = ub;
      }
      d->sweep_count++;
      d->t_pos = d->t_neg = 0;
    }
    __syncthreads();
    int q;
    for (q = 1; q <= swp_num; ++q) {
      for (int pass = 0; pass < 2; ++pass) {
        flag_list(pass, S);
        if (threadIdx.x == 0) walk(pass, S.ub, S);
        __syncthreads();
      }
      if (threadIdx.x == 0) d->pre_count++;
      double pmin, pu;
      pressure_data_par(pmin, pu, S);
      const double rmin = rho_min_par(S);
      if (pmin > epsi && rmin > epsi) break;
    }
    if (threadIdx.x == 0) {
      const long long k = d->sweep_count - 1;
      if (q > swp_num) {
        q = swp_num;
        d->fail_count++;
      }
      if (k < d->track_cap) {
        d->tracks[k] = q;
        d->tracks[d->track_cap + k] = (int)d->t_neg;
        d->tracks[2 * d->track_cap + k] = (int)d->t_pos;
      }
    }
    __syncthreads();
  }
  // apply_sweep.m, block-cooperative
  __device__ void apply_par(int swp_num, SweepShared& S) {
    if (rho_min_par(S) <= 1e-13) {
      if (threadIdx.x == 0) scalar_pos();
      __syncthreads();
    }
    double pmin, pu;
    pressure_data_par(pmin, pu, S);
    if (pmin <= 1e-13 && pu > 0) {
      if (threadIdx.x == 0) scalar_pos();
      __syncthreads();
      pressure_data_par(pmin, pu, S);
      if (pu > 1e-13) swp_alg_par(swp_num, S);
    }
  }
  // apply_sweep.m
  __device__ void apply(int swp_num) {
    if (rho_min() <= 1e-13) scalar_pos();
    double pmin, pu;
    pressure_data(pmin, pu);
    if (pmin <= 1e-13 && pu > 0) {
      scalar_pos();
      pressure_data(pmin, pu);
      if (pu > 1e-13) swp_alg(swp_num);
    }
  }
};

__global__ void __launch_bounds__(MT, 1)
    k_matlab1d(Params p, double* __restrict__ u, double* __restrict__ wk, DevScalars* d,
               long long max_steps, int per, int sweeping, int swp_num, double cfl) {
  __shared__ double sh[32];
  __shared__ double s_l;
  __shared__ int s_go;
  __shared__ SweepShared ssw;
  const int n = p.g.nx;
  const int64_t P = p.g.plane;
  const Ctx c{n, per, p.gamma - 1};
  const Work w = carve(wk, n);
  const double g = p.gamma, h = p.dx;
  long long steps = 0;
  for (;;) {
    if (threadIdx.x == 0)
      s_go = (d->time < p.time_terminal) && (steps < max_steps) && d->error == 0;
    __syncthreads();
    if (!s_go) break;
    // eigenvalues of the cell states and the time step (:217-252)
    const double qnan = __longlong_as_double(0x7ff8000000000000ll);
    double a[3] = {qnan, qnan, qnan};
    for (int i = 1 + threadIdx.x; i <= n; i += MT) {
      const double ro = u[i + 2], m = u[P + i + 2], E = u[2 * P + i + 2];
      const double v = m / ro;
      const double pr = E * c.g1 - 1. / 2. * ro * (v * v) * c.g1;
      const double cs = sqrt((g * pr) / ro);
      a[0] = fmax(a[0], fabs(v - cs));
      a[1] = fmax(a[1], fabs(v));
      a[2] = fmax(a[2], fabs(v + cs));
    }
    block_max3(a, sh);
    if (threadIdx.x == 0) {
      const double alpha = fmax(fmax(a[0], a[1]), a[2]);
      double k = cfl * h / alpha;
      if (p.time_terminal - d->time < k) k = p.time_terminal - d->time;
      d->alphamax = alpha;
      d->dt = k;
      s_l = k / h;
    }
    __syncthreads();
    const double l = s_l;
    for (int stage = 1; stage <= 3; ++stage) {
      if (stage == 1) fluxes(c, u, (int)P, 3, w, sh);
      else fluxes(c, w.uh, n, 0, w, sh);
      for (int i = 1 + threadIdx.x; i <= n; i += MT)
        for (int r = 0; r < 3; ++r) {
          const double fp = w.fP[r * n + i - 1];
          const double fm = i >= 2 ? w.fP[r * n + i - 2] : (per ? w.fP[r * n + n - 1] : w.fM0[r]);
          const double dd = l * (fp - fm);
          const double ui = u[r * P + i + 2];
          double& o = w.uh[r * n + i - 1];
          if (stage == 1) o = ui - dd;
          else if (stage == 2) o = 3. / 4. * ui + 1. / 4. * (o - dd);
          else o = 1. / 3. * ui + 2. / 3. * (o - dd);
        }
      __syncthreads();
      if (sweeping) {
        Sweep sw{w.uh, n, 1. * 1. / n, d};
        if (n - 1 <= SW_CAP) {
          sw.apply_par(swp_num, ssw);
        } else if (threadIdx.x == 0) {
          sw.apply(swp_num);
        }
      }
      __syncthreads();
    }
    // u = uHold; the ghosts take the padding of the new state
    for (int J = 1 + threadIdx.x; J <= n + 6; J += MT) {
      const int i = pad_src(c, J);
      for (int r = 0; r < 3; ++r) u[r * P + J - 1] = w.uh[r * n + i - 1];
    }
    if (threadIdx.x == 0) {
      d->time = d->time + d->dt;
      d->steps++;
    }
    ++steps;
    __syncthreads();
  }
}

}  // namespace

int64_t matlab1d_workspace(int n) { return 6 * (int64_t)n + 4 + 12 * ((int64_t)n + 8); }

cudaError_t launch_matlab1d(const Params& p, double* u, double* wk, DevScalars* d,
                            long long max_steps, int periodic, int sweeping, int swp_num,
                            double cfl, cudaStream_t s) {
  k_matlab1d<<<1, MT, 0, s>>>(p, u, wk, d, max_steps, periodic, sweeping, swp_num, cfl);
  return cudaGetLastError();
}

}  // namespace swfd
