/* swfd_serve.c -- a C host request loop over the library's batch API.
 *
 * A stream of independent Euler solves arrives with Poisson inter-arrival
 * times: the vortex (ex3_vortex_accuracy_2d), the point-energy problem
 * (ex4_sedov_2d, shortened to T = 0.02) and the Mach 5.09 shock diffraction
 * (ex6_shock_diffraction, shortened to T = 0.05), drawn uniformly.  Vortex
 * and point-energy requests go to an FP32-bulk batch, the shock diffraction
 * to an FP64 batch.  Each batch is driven by its own host thread: it admits
 * the requests that have arrived while a slot and enough of its HBM budget
 * are free (first come, first served), advances every running request
 * together by --chunk SSP-RK3 steps per graph launch, and reads back,
 * records and releases the finished ones -- continuous batching.  The
 * program prints one JSON line with the time-to-solution percentiles and the
 * aggregate cell-updates/s; with --check it solves some finished requests
 * again alone (swfd_create / swfd_run) and counts those whose final state is
 * the same to the last bit.
 *
 * usage: swfd_serve [--requests N] [--rate HZ] [--seed S] [--slots K]
 *                   [--chunk STEPS] [--small] [--check M] [--device D]
 */
#define _POSIX_C_SOURCE 200809L
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "swfd.h"

typedef struct {
  double arrival;        /* s after the start */
  swfd_config cfg;
  int batch;             /* 0: FP32-bulk, 1: FP64 */
  double latency;        /* arrival to result on the host, s */
  int32_t status;
  int64_t updates;       /* interior cells x 3 stages x steps */
  double* u;             /* final state, kept for --check */
  int done;
} request;

typedef struct {
  swfd_batch* b;
  int which;
  request* req;
  int nreq;
  int64_t chunk;
  double t0;
  int64_t launches;
  int error;
} driver;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static uint64_t rng_state;
static uint64_t rng_next(void) { /* splitmix64 */
  uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
static double rng_unit(void) { return ((double)(rng_next() >> 11) + 1.0) / 9007199254740993.0; }

static int64_t state_len(const swfd_config* c) {
  return c->problem == SWFD_PROBLEM_SEDOV_1D
             ? 3 * (int64_t)(c->nx + 6)
             : 4 * (int64_t)(c->nx + 6) * (int64_t)(c->ny + 6);
}

static void draw(request* r, int small) {
  const int kind = (int)(rng_next() % 3);
  swfd_config* c = &r->cfg;
  if (kind == 0) {
    static const int n_full[] = {45, 90, 180, 360}, n_small[] = {45, 64};
    const int n = small ? n_small[rng_next() % 2] : n_full[rng_next() % 4];
    swfd_config_default(c, SWFD_PROBLEM_VORTEX_2D);
    c->nx = c->ny = n;
  } else if (kind == 1) {
    const int lo = small ? 40 : 128, hi = small ? 80 : 640;
    swfd_config_default(c, SWFD_PROBLEM_SEDOV_2D);
    c->nx = c->ny = lo + (int)(rng_next() % (uint64_t)(hi - lo + 1));
    c->time_terminal = small ? 0.005 : 0.02;
  } else {
    static const int t_full[] = {20, 40, 60, 80}, t_small[] = {12, 20};
    const int total = small ? t_small[rng_next() % 2] : t_full[rng_next() % 4];
    swfd_config_default(c, SWFD_PROBLEM_SHOCK_DIFFRACTION);
    c->total = total;
    c->nx = c->cut_x * (13 * total / c->cut_x);
    c->ny = c->cut_y * (11 * total / c->cut_y);
    c->time_terminal = small ? 0.01 : 0.05;
  }
  /* FP32-bulk is accepted for the vortex and the point energy (relative L1
   * density error below 1e-6); the shock diffraction stays FP64 */
  r->batch = kind == 2;
  c->precision = r->batch ? SWFD_PRECISION_FP64 : SWFD_PRECISION_FP32_BULK;
}

static void* drive(void* arg) {
  driver* d = (driver*)arg;
  int next = 0, finished = 0, mine = 0;
  for (int k = 0; k < d->nreq; ++k) mine += d->req[k].batch == d->which;
  int64_t ids[64];
  int32_t sts[64];
  while (finished < mine) {
    const double t = now_s() - d->t0;
    int32_t running = 0, free_slots = 0;
    int64_t free_bytes = 0;
    swfd_batch_info(d->b, &running, &free_slots, &free_bytes);
    /* admit what has arrived, first come first served */
    while (next < d->nreq) {
      request* r = &d->req[next];
      if (r->batch != d->which) {
        ++next;
        continue;
      }
      if (r->arrival > t) break;
      swfd_status st = swfd_batch_admit(d->b, &r->cfg, next);
      if (st == SWFD_ERR_OOM && running > 0) break; /* wait for releases */
      if (st != SWFD_OK) { /* refused, or larger than the whole empty batch */
        r->status = st, r->done = 1, r->latency = now_s() - d->t0 - r->arrival;
        ++finished, ++next;
        continue;
      }
      ++next;
      ++running;
    }
    if (!running) {
      if (finished < mine) {
        struct timespec ts = {0, 1000000};
        nanosleep(&ts, NULL);
      }
      continue;
    }
    int64_t steps = 0;
    if (swfd_batch_run(d->b, d->chunk, &steps) != SWFD_OK) {
      d->error = 1;
      return NULL;
    }
    d->launches++;
    int32_t n = 0;
    do {
      swfd_batch_poll(d->b, ids, sts, 64, &n);
      for (int k = 0; k < n; ++k) {
        request* r = &d->req[ids[k]];
        r->u = (double*)malloc((size_t)state_len(&r->cfg) * sizeof(double));
        double tt = 0;
        int64_t st_steps = 0;
        swfd_batch_download(d->b, ids[k], r->u, &tt);
        swfd_batch_progress(d->b, ids[k], &tt, &st_steps);
        r->latency = now_s() - d->t0 - r->arrival;
        r->status = sts[k];
        r->updates = (int64_t)r->cfg.nx * r->cfg.ny * 3 * st_steps;
        r->done = 1;
        swfd_batch_release(d->b, ids[k]);
        ++finished;
      }
    } while (n == 64);
  }
  return NULL;
}

static int cmp_double(const void* a, const void* b) {
  const double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* linear interpolation between closest ranks (numpy's default) */
static double percentile(const double* v, int n, double q) {
  if (n == 0) return NAN;
  const double pos = q / 100.0 * (n - 1);
  const int lo = (int)floor(pos), hi = lo + 1 < n ? lo + 1 : lo;
  return v[lo] + (v[hi] - v[lo]) * (pos - lo);
}

int main(int argc, char** argv) {
  int nreq = 24, slots = 32, small = 0, check = 0, device = 0;
  double rate = 50.0;
  int64_t chunk = 4;
  uint64_t seed = 20261204;
  for (int k = 1; k < argc; ++k) {
    const char* a = argv[k];
    const char* v = k + 1 < argc ? argv[k + 1] : "0";
    if (!strcmp(a, "--requests")) nreq = atoi(v), ++k;
    else if (!strcmp(a, "--rate")) rate = atof(v), ++k;
    else if (!strcmp(a, "--seed")) seed = strtoull(v, NULL, 10), ++k;
    else if (!strcmp(a, "--slots")) slots = atoi(v), ++k;
    else if (!strcmp(a, "--chunk")) chunk = atoll(v), ++k;
    else if (!strcmp(a, "--check")) check = atoi(v), ++k;
    else if (!strcmp(a, "--device")) device = atoi(v), ++k;
    else if (!strcmp(a, "--small")) small = 1;
    else {
      fprintf(stderr, "unknown argument %s\n", a);
      return 2;
    }
  }
  if (nreq < 1 || nreq > 100000 || slots < 1 || chunk < 1 || !(rate > 0)) {
    fprintf(stderr, "bad arguments\n");
    return 2;
  }
  rng_state = seed;
  request* req = (request*)calloc((size_t)nreq, sizeof(request));
  double t = 0;
  for (int k = 0; k < nreq; ++k) {
    t += -log(rng_unit()) / rate;
    req[k].arrival = t;
    draw(&req[k], small);
    req[k].cfg.device = device;
  }
  swfd_batch* b[2] = {NULL, NULL};
  for (int w = 0; w < 2; ++w) {
    swfd_batch_config bc;
    swfd_batch_config_default(&bc);
    bc.max_slots = w == 0 ? slots : (slots / 4 > 4 ? slots / 4 : 4);
    bc.max_nx = w == 0 ? 640 : 1040;
    bc.max_ny = w == 0 ? 640 : 880;
    bc.precision = w == 0 ? SWFD_PRECISION_FP32_BULK : SWFD_PRECISION_FP64;
    bc.ubar_mode = SWFD_UBAR_SEQUENTIAL; /* the single-instance u_bar: results equal alone */
    bc.device = device;
    if (swfd_batch_create(&bc, &b[w]) != SWFD_OK) {
      char m[512];
      swfd_last_error(NULL, m, sizeof m);
      fprintf(stderr, "swfd_batch_create: %s\n", m);
      return 1;
    }
  }
  driver d[2];
  pthread_t th[2];
  const double t0 = now_s();
  for (int w = 0; w < 2; ++w) {
    d[w] = (driver){b[w], w, req, nreq, chunk, t0, 0, 0};
    pthread_create(&th[w], NULL, drive, &d[w]);
  }
  for (int w = 0; w < 2; ++w) pthread_join(th[w], NULL);
  const double wall = now_s() - t0;
  for (int w = 0; w < 2; ++w) swfd_batch_destroy(b[w]);

  double* lat = (double*)malloc((size_t)nreq * sizeof(double));
  int nd = 0, failed = 0, per[2] = {0, 0};
  double upd = 0;
  for (int k = 0; k < nreq; ++k) {
    if (!req[k].done) continue;
    lat[nd++] = req[k].latency;
    failed += req[k].status != 0;
    upd += (double)req[k].updates;
    per[req[k].batch]++;
  }
  qsort(lat, (size_t)nd, sizeof(double), cmp_double);

  /* --check: the first M finished requests of each batch, solved alone */
  int compared = 0, equal = 0;
  for (int w = 0; w < 2 && check > 0; ++w) {
    int m = 0;
    for (int k = 0; k < nreq && m < check; ++k) {
      request* r = &req[k];
      if (!r->done || r->batch != w || r->status != 0 || !r->u) continue;
      ++m;
      swfd_handle* h = NULL;
      if (swfd_create(&r->cfg, &h) != SWFD_OK) continue;
      int64_t steps = 0;
      swfd_init_problem(h);
      swfd_run(h, 0, &steps);
      const int64_t len = state_len(&r->cfg);
      double* u = (double*)malloc((size_t)len * sizeof(double));
      swfd_download_state(h, u);
      ++compared;
      equal += memcmp(u, r->u, (size_t)len * sizeof(double)) == 0;
      free(u);
      swfd_destroy(h);
    }
  }
  printf("{\"requests\": %d, \"finished\": %d, \"failed\": %d, \"fp32_bulk_requests\": %d, "
         "\"fp64_requests\": %d, \"p50_s\": %.6f, \"p99_s\": %.6f, \"max_s\": %.6f, "
         "\"wall_s\": %.6f, \"cell_updates\": %.0f, \"value\": %.6e, \"unit\": \"cell-updates/s\", "
         "\"graph_launches\": %lld, \"errors\": %d, \"check\": {\"compared\": %d, \"equal\": %d}}\n",
         nreq, nd, failed, per[0], per[1], percentile(lat, nd, 50), percentile(lat, nd, 99),
         nd ? lat[nd - 1] : NAN, wall, upd, wall > 0 ? upd / wall : 0.0,
         (long long)(d[0].launches + d[1].launches), d[0].error + d[1].error, compared, equal);
  for (int k = 0; k < nreq; ++k) free(req[k].u);
  free(req);
  free(lat);
  return (d[0].error || d[1].error || nd != nreq) ? 1 : 0;
}
