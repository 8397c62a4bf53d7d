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

__device__ __forceinline__ int64_t npos(const Geom& g) {
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

}  // namespace swfd
