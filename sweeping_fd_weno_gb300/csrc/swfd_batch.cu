// swfd_batch.cu -- the batched engine: many independent 2D problem instances
// resident on one GPU, advanced together.  Every kernel of a stage is one
// launch over all instances (the slot table is read on the device), the flux
// kernel is one persistent launch whose chunk counter spans all instances,
// and a whole run (WHILE some instance is running: three stages with their
// conditional sweeps, then each instance's own time test) is one CUDA graph.
// Admission, completion and retirement happen between graph launches by
// rewriting the slot table, so the graph never changes: this is what the
// continuous-batching serving loop drives.
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "swfd_graph.h"
#include "swfd_internal.h"

using namespace swfd;

namespace {

struct SlotHost {
  int state = 0;  // 0 free, 1 running, 2 finished (not yet polled), 3 polled
  int64_t id = -1;
  swfd_config cfg{};
  Params p{};
  void* mem = nullptr;   // state, split, roe, flux planes and sweep scratch
  DevScalars* dsc = nullptr;
  int* tracks = nullptr;
  int64_t track_cap = 0;
  size_t bytes = 0;
  int status = 0;
  DevScalars last{};     // device scalars at the last synchronisation
};

size_t a256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

struct swfd_batch {
  swfd_batch_config cfg{};
  cudaStream_t stream = nullptr;
  cudaStream_t cap[4] = {};
  std::vector<SlotHost> slots;
  std::vector<BatchSlot> tab;
  BatchSlot* d_tab = nullptr;
  BatchCtl* d_ctl = nullptr;
  BatchCtl* h_ctl = nullptr;
  long long* d_prefix = nullptr;
  std::vector<long long> prefix;
  long long* d_tprefix = nullptr;  // cell-tile prefix of the per-cell kernels
  std::vector<long long> tprefix;
  long long* d_s32prefix = nullptr;  // the fused FP32-bulk stage's tile + ghost-chunk prefix
  std::vector<long long> s32prefix;
  // FP32-bulk: this run's running slots are all 2D without rank segments,
  // limiter or binary128 literals: the graph with the fused stage
  bool fast = false;
  int tile_cells = 2048;           // cells per tile (swfd_batch_autotune picks it)
  DevScalars* d_dsc = nullptr;  // one DevScalars per slot, contiguous: one read-back per run
  DevScalars* h_dsc = nullptr;  // pinned mirror
  cudaGraphExec_t g_run = nullptr;
  cudaGraphExec_t g_fast = nullptr;  // the same loop with the fused FP32-bulk stage
  double* d_stage = nullptr;
  size_t stage_bytes = 0;
  int64_t pool_bytes = 0, used_bytes = 0;
  long long max_cell = 0;
  std::string last_error;
  std::mutex mu;  // the serving API may be called from several host threads
};

namespace {

swfd_status bfail(swfd_batch* b, swfd_status st, const std::string& m) {
  if (b) b->last_error = m;
  swfd::set_last_error(m);
  return st;
}

#define BCU(b, call)                                                                       \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return bfail((b), e_ == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA,    \
                   std::string(#call) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

// plane strides of a slot, in elements, rounded so that every plane starts
// on a 256-byte boundary: the state and Roe planes (g) and the split and
// flux planes (sg: one copy per rank segment for ex6, else sg == g)
size_t state_plane_elems(const Params& p) { return a256((size_t)p.g.plane * sizeof(double)) / 8; }
size_t seg_plane_elems(const Params& p) { return a256((size_t)p.sg.plane * sizeof(double)) / 8; }

size_t seg_alpha_elems(const Params& p) {
  return p.seg_alpha ? state_plane_elems(p) + (size_t)p.g.LJ * p.cut_x + (size_t)p.g.LI * p.cut_y +
                           (size_t)12 * (6 * p.total + 2)
                     : 0;
}

// device footprint of one instance
size_t slot_bytes(const Params& p, int fp32) {
  const size_t pe = state_plane_elems(p), se = seg_plane_elems(p), ts = fp32 ? 4 : 8;
  const int nc = p.g.nc;
  return 3 * nc * pe * 8 + a256(4 * nc * se * ts) + a256(8 * pe * ts) + a256(4 * nc * se * ts) +
         a256(sweep_scratch_bytes(p)) + a256(seg_alpha_elems(p) * 8);
}

BatchLaunch launch_desc(swfd_batch* b) {
  BatchLaunch L;
  L.tab = b->d_tab;
  L.ctl = b->d_ctl;
  L.prefix = b->d_prefix;
  L.tprefix = b->d_tprefix;
  L.s32prefix = b->d_s32prefix;
  L.n_slots = b->cfg.max_slots;
  L.max_cell = b->max_cell;
  L.fp32 = b->cfg.precision == SWFD_PRECISION_FP32_BULK;
  L.ubar_tree = b->cfg.ubar_mode == SWFD_UBAR_TREE;
  L.segmented = 1;
  return L;
}

// WHILE (some slot runs and steps < limit) { stage 1..3 with conditional
// sweeps and bc; per-slot time advance }; fast: the FP32-bulk fused stage
// (for slots that are all 2D without rank segments, limiter or binary128
// literals).  An FP64 form of the fast graph with the lane-pair flux kernel
// was measured slower than kb_flux<double> here (2.21e8 against 2.52e8
// cell-updates/s on the 256-instance mix) and is not built.
swfd_status build_run_graph(swfd_batch* b, bool fast) {
  Builder bd;
  bd.cap = b->cap;
  bd.max_depth = 3;
  const BatchLaunch L = launch_desc(b);
  const bool fused = fast;
  cudaStream_t s = b->cap[0];
  BCU(b, cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
  cudaStreamCaptureStatus cs;
  bd.ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &bd.root, nullptr, nullptr, nullptr));
  B_OK(bd, cudaMemsetAsync(&b->d_ctl->steps, 0, sizeof(long long), s));
  cudaGraphConditionalHandle hr = bd.handle();
  B_OK(bd, launch_batch_run_cond(hr, L, 0, s));
  bd.cond(s, cudaGraphCondTypeWhile, hr, [&](cudaStream_t sb) {
    const int in_of[3] = {0, 1, 2}, out_of[3] = {1, 2, 0};
    for (int k = 1; k <= 3; ++k) {
      const int in = in_of[k - 1], out = out_of[k - 1];
      cudaGraphConditionalHandle hs = bd.handle();
      if (fused) B_OK(bd, launch_batch_stage32(L, k, in, out, hs, sb));
      else B_OK(bd, launch_batch_stage(L, k, in, out, hs, sb));
      bd.cond(sb, cudaGraphCondTypeIf, hs, [&](cudaStream_t sw) {
        B_OK(bd, launch_batch_sweep_head(L, out, sw));
        cudaGraphConditionalHandle hq = bd.handle();
        B_OK(bd, launch_batch_sweep_cond(L, hq, sw));
        bd.cond(sw, cudaGraphCondTypeWhile, hq, [&](cudaStream_t sq) {
          B_OK(bd, launch_batch_sweep_iter(L, out, hq, sq));
        });
      });
      B_OK(bd, launch_batch_bc(L, out, sb));
    }
    B_OK(bd, launch_batch_time_advance(L, sb));
    B_OK(bd, launch_batch_run_cond(hr, L, 1, sb));
  });
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(s, &g);
  if (bd.err != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return bfail(b, SWFD_ERR_CUDA, std::string("batch graph capture: ") +
                                       cudaGetErrorString(bd.err != cudaSuccess ? bd.err : e2));
  }
  cudaError_t e3 = cudaGraphInstantiate(fast ? &b->g_fast : &b->g_run, g, 0);
  cudaGraphDestroy(g);
  if (e3 != cudaSuccess)
    return bfail(b, SWFD_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e3));
  return SWFD_OK;
}

int find_slot(swfd_batch* b, int64_t id) {
  for (size_t k = 0; k < b->slots.size(); ++k)
    if (b->slots[k].state != 0 && b->slots[k].id == id) return (int)k;
  return -1;
}

swfd_status free_slot(swfd_batch* b, int k) {
  SlotHost& sh = b->slots[k];
  cudaFree(sh.mem);
  cudaFree(sh.tracks);
  b->used_bytes -= (int64_t)sh.bytes;
  sh = SlotHost();
  b->tab[k] = BatchSlot{};
  BCU(b, cudaMemcpyAsync(b->d_tab + k, &b->tab[k], sizeof(BatchSlot), cudaMemcpyHostToDevice,
                         b->stream));
  return SWFD_OK;
}

swfd_status ensure_slot_tracks(swfd_batch* b, int k, int64_t extra) {
  SlotHost& sh = b->slots[k];
  int64_t need = sh.last.sweep_count + extra;
  if (need <= sh.track_cap) return SWFD_OK;
  int64_t cap = std::max<int64_t>(need, 2 * sh.track_cap + 1024);
  int* nt = nullptr;
  BCU(b, cudaMalloc(&nt, 3 * cap * sizeof(int)));
  BCU(b, cudaMemsetAsync(nt, 0, 3 * cap * sizeof(int), b->stream));
  for (int c = 0; c < 3 && sh.tracks; ++c)
    BCU(b, cudaMemcpyAsync(nt + c * cap, sh.tracks + c * sh.track_cap, sh.track_cap * sizeof(int),
                           cudaMemcpyDeviceToDevice, b->stream));
  long long lc = cap;
  BCU(b, cudaMemcpyAsync(&sh.dsc->tracks, &nt, sizeof(int*), cudaMemcpyHostToDevice, b->stream));
  BCU(b, cudaMemcpyAsync(&sh.dsc->track_cap, &lc, sizeof(long long), cudaMemcpyHostToDevice,
                         b->stream));
  BCU(b, cudaStreamSynchronize(b->stream));
  cudaFree(sh.tracks);
  sh.tracks = nt;
  sh.track_cap = cap;
  return SWFD_OK;
}

swfd_status status_of(int err_bits) {
  if (err_bits & ERR_BIT_CHECK) return SWFD_ERR_SWEEP_CHECK;
  if (err_bits & ERR_BIT_PUBAR) return SWFD_ERR_PUBAR_NONPOS;
  if (err_bits & ERR_BIT_NOCONV) return SWFD_ERR_SWEEP_NOCONV;
  if (err_bits) return SWFD_ERR_NONFINITE;
  return SWFD_OK;
}

}  // namespace

extern "C" {

swfd_status swfd_batch_config_default(swfd_batch_config* c) {
  if (!c) return SWFD_ERR_INVALID;
  memset(c, 0, sizeof(*c));
  c->max_slots = 256;
  c->max_nx = 640;
  c->max_ny = 640;
  c->precision = SWFD_PRECISION_FP32_BULK;
  c->ubar_mode = SWFD_UBAR_TREE;
  c->device = 0;
  c->pool_bytes = 0;
  return SWFD_OK;
}

swfd_status swfd_batch_create(const swfd_batch_config* cfg, swfd_batch** out) {
  if (!cfg || !out) return bfail(nullptr, SWFD_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (cfg->max_slots < 1 || cfg->max_slots > 65535 || cfg->max_nx < 8 || cfg->max_ny < 8)
    return bfail(nullptr, SWFD_ERR_INVALID, "max_slots in [1, 65535] and max_nx, max_ny >= 8");
  if (cfg->precision != SWFD_PRECISION_FP64 && cfg->precision != SWFD_PRECISION_FP32_BULK)
    return bfail(nullptr, SWFD_ERR_INVALID, "unknown precision");
  if (cfg->ubar_mode != SWFD_UBAR_SEQUENTIAL && cfg->ubar_mode != SWFD_UBAR_TREE)
    return bfail(nullptr, SWFD_ERR_INVALID, "unknown ubar_mode");
  swfd_batch* b = new swfd_batch();
  b->cfg = *cfg;
  auto bad = [&](cudaError_t e) {
    std::string m = std::string("swfd_batch_create: ") + cudaGetErrorString(e);
    swfd_batch_destroy(b);
    return bfail(nullptr, e == cudaErrorMemoryAllocation ? SWFD_ERR_OOM : SWFD_ERR_CUDA, m);
  };
  cudaError_t e;
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess) return bad(e);
  if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) return bad(e);
  for (int k = 0; k < 4; ++k)
    if ((e = cudaStreamCreateWithFlags(&b->cap[k], cudaStreamNonBlocking)) != cudaSuccess)
      return bad(e);
  const int n = cfg->max_slots;
  b->slots.resize(n);
  b->tab.assign(n, BatchSlot{});
  b->prefix.assign(n + 1, 0);
  b->tprefix.assign(n + 1, 0);
  b->s32prefix.assign(n + 1, 0);
  b->max_cell = (long long)(cfg->max_nx + 6) * (cfg->max_ny + 6);
  b->stage_bytes = (size_t)4 * b->max_cell * sizeof(double);
  if ((e = cudaMalloc(&b->d_tab, n * sizeof(BatchSlot))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_ctl, sizeof(BatchCtl))) != cudaSuccess) return bad(e);
  if ((e = cudaMallocHost(&b->h_ctl, sizeof(BatchCtl))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_prefix, (n + 1) * sizeof(long long))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_tprefix, (n + 1) * sizeof(long long))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_s32prefix, (n + 1) * sizeof(long long))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_stage, b->stage_bytes)) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&b->d_dsc, n * sizeof(DevScalars))) != cudaSuccess) return bad(e);
  if ((e = cudaMallocHost(&b->h_dsc, n * sizeof(DevScalars))) != cudaSuccess) return bad(e);
  if ((e = cudaMemcpyAsync(b->d_tab, b->tab.data(), n * sizeof(BatchSlot), cudaMemcpyHostToDevice,
                           b->stream)) != cudaSuccess)
    return bad(e);
  if ((e = cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchCtl), b->stream)) != cudaSuccess) return bad(e);
  if ((e = cudaMemsetAsync(b->d_prefix, 0, (n + 1) * sizeof(long long), b->stream)) != cudaSuccess)
    return bad(e);
  if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return bad(e);
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  b->pool_bytes = cfg->pool_bytes > 0 ? cfg->pool_bytes : (int64_t)(0.8 * (double)fr);
  const bool f32 = cfg->precision == SWFD_PRECISION_FP32_BULK;
  if (f32 && (e = stage32_setup()) != cudaSuccess) return bad(e);
  if (build_run_graph(b, false) != SWFD_OK || (f32 && build_run_graph(b, true) != SWFD_OK)) {
    std::string m = b->last_error;
    swfd_batch_destroy(b);
    return bfail(nullptr, SWFD_ERR_CUDA, m);
  }
  *out = b;
  return SWFD_OK;
}

swfd_status swfd_batch_destroy(swfd_batch* b) {
  if (!b) return SWFD_OK;
  cudaSetDevice(b->cfg.device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& sh : b->slots) {
    cudaFree(sh.mem);
    cudaFree(sh.tracks);
  }
  if (b->g_run) cudaGraphExecDestroy(b->g_run);
  if (b->g_fast) cudaGraphExecDestroy(b->g_fast);
  cudaFree(b->d_tab);
  cudaFree(b->d_ctl);
  cudaFree(b->d_prefix);
  cudaFree(b->d_tprefix);
  cudaFree(b->d_s32prefix);
  cudaFree(b->d_stage);
  cudaFree(b->d_dsc);
  if (b->h_ctl) cudaFreeHost(b->h_ctl);
  if (b->h_dsc) cudaFreeHost(b->h_dsc);
  for (int k = 0; k < 4; ++k)
    if (b->cap[k]) cudaStreamDestroy(b->cap[k]);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SWFD_OK;
}

swfd_status swfd_batch_admit(swfd_batch* b, const swfd_config* cfg, int64_t request_id) {
  if (!b || !cfg) return bfail(b, SWFD_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(b->mu);
  std::string err;
  swfd_config c = *cfg;
  c.precision = b->cfg.precision;
  c.ubar_mode = SWFD_UBAR_SEQUENTIAL;  // validated as the single-instance path
  swfd_status st = check_config(c, err);
  if (st != SWFD_OK) return bfail(b, st, err);
  if (c.literals != SWFD_LITERALS_DOUBLE)
    return bfail(b, SWFD_ERR_UNSUPPORTED, "the batched engine runs the binary64 literals");
  if (c.problem == SWFD_PROBLEM_SEDOV_1D || c.problem == SWFD_PROBLEM_MATLAB_1D)
    return bfail(b, SWFD_ERR_UNSUPPORTED, "the batched engine holds 2D problems");
  if (c.problem == SWFD_PROBLEM_DETONATION)
    return bfail(b, SWFD_ERR_UNSUPPORTED, "the batched engine holds the four-component problems");
  if (c.use_limiter == 1)
    return bfail(b, SWFD_ERR_UNSUPPORTED,
                 "the batched engine runs the sweeping form (use_limiter 0 or 2)");
  if (c.nx > b->cfg.max_nx || c.ny > b->cfg.max_ny)
    return bfail(b, SWFD_ERR_INVALID, "grid larger than the batch's max_nx x max_ny");
  if (find_slot(b, request_id) >= 0) return bfail(b, SWFD_ERR_INVALID, "request id in use");
  Params p;
  st = make_params(c, p, err);
  if (st != SWFD_OK) return bfail(b, st, err);
  int k = -1;
  for (size_t s = 0; s < b->slots.size(); ++s)
    if (b->slots[s].state == 0) {
      k = (int)s;
      break;
    }
  const int fp32 = b->cfg.precision == SWFD_PRECISION_FP32_BULK;
  const size_t bytes = slot_bytes(p, fp32);
  if (k < 0) return bfail(b, SWFD_ERR_OOM, "no free slot");
  if (b->used_bytes + (int64_t)bytes > b->pool_bytes)
    return bfail(b, SWFD_ERR_OOM, "HBM budget of the batch exhausted");
  BCU(b, cudaSetDevice(b->cfg.device));
  SlotHost& sh = b->slots[k];
  BCU(b, cudaMalloc(&sh.mem, bytes));
  sh.bytes = bytes;
  b->used_bytes += (int64_t)bytes;
  sh.track_cap = 1024;
  BCU(b, cudaMalloc(&sh.tracks, 3 * sh.track_cap * sizeof(int)));
  BCU(b, cudaMemsetAsync(sh.tracks, 0, 3 * sh.track_cap * sizeof(int), b->stream));
  // carve the slot's buffers
  const size_t pe = state_plane_elems(p), se = seg_plane_elems(p), ts = fp32 ? 4 : 8;
  const int nc = p.g.nc;
  char* cptr = (char*)sh.mem;
  BatchSlot bs{};
  for (int s = 0; s < 3; ++s) {
    bs.st[s] = (double*)cptr;
    cptr += nc * pe * 8;
  }
  bs.split = cptr;
  cptr += a256(4 * nc * se * ts);
  bs.roe = cptr;
  cptr += a256(8 * pe * ts);
  bs.flux = cptr;
  cptr += a256(4 * nc * se * ts);
  bs.sweep_scratch = cptr;
  cptr += a256(sweep_scratch_bytes(p));
  sh.dsc = b->d_dsc + k;
  bs.dsc = sh.dsc;
  bs.p = p;
  bs.p.g.plane = (int64_t)pe;
  bs.p.sg.plane = (int64_t)se;
  if (p.seg_alpha) {
    bs.p.alpha_plane = (double*)cptr;
    bs.p.seg_ax = bs.p.alpha_plane + pe;
    bs.p.seg_ay = bs.p.seg_ax + (size_t)p.g.LJ * p.cut_x;
    bs.p.wall_save = bs.p.seg_ay + (size_t)p.g.LI * p.cut_y;
  }
  bs.ncell = (long long)p.g.LI * p.g.LJ;
  bs.chunks_x = (flux_faces_x(p) + 31) / 32;
  bs.chunks = bs.chunks_x + (flux_faces_y(p) + 31) / 32;
  bs.use_limiter = c.use_limiter;
  bs.swp_num = c.swp_num;
  bs.stop_on_fail = p.stop_sweep;
  bs.active = 0;  // set once the state is in place
  // initial data
  std::vector<double> u((size_t)nc * p.g.LI * p.g.LJ);
  init_host_state(p, c, u.data());
  BCU(b, cudaMemcpyAsync(b->d_stage, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice,
                         b->stream));
  BCU(b, launch_fortran_to_soa(bs.p, b->d_stage, bs.st[0], b->stream));
  if (p.problem != SWFD_PROBLEM_SHOCK_DIFFRACTION)  // ex6 starts from initdata
    BCU(b, launch_bc(bs.p, bs.st[0], b->stream));
  DevScalars d{};
  d.tracks = sh.tracks;
  d.track_cap = sh.track_cap;
  d.t_end = c.time_terminal;
  BCU(b, cudaMemcpyAsync(sh.dsc, &d, sizeof(DevScalars), cudaMemcpyHostToDevice, b->stream));
  bs.active = 1;
  b->tab[k] = bs;
  BCU(b, cudaMemcpyAsync(b->d_tab + k, &b->tab[k], sizeof(BatchSlot), cudaMemcpyHostToDevice,
                         b->stream));
  BCU(b, cudaStreamSynchronize(b->stream));
  sh.state = 1;
  sh.id = request_id;
  sh.cfg = c;
  sh.p = bs.p;
  sh.last = d;
  sh.status = 0;
  return SWFD_OK;
}

namespace {
// the running slots' work plan: flux-chunk and cell-tile prefixes and the
// batch scalars of a launch of up to max_steps steps
swfd_status upload_plan(swfd_batch* b, int64_t max_steps) {
  const int n = b->cfg.max_slots;
  int running = 0;
  long long chunks = 0, tiles = 0, items = 0;
  // the fused FP32-bulk stage when every running slot takes it (2D, no rank
  // segments, no limiter, binary64 literals) and SWFD_FP32_STAGE is not
  // "split"
  const char* fs = getenv("SWFD_FP32_STAGE");
  bool fused = b->g_fast != nullptr && !(fs && strcmp(fs, "split") == 0);
  for (int k = 0; k < n; ++k) {
    b->prefix[k] = chunks;
    b->tprefix[k] = tiles;
    b->s32prefix[k] = items;
    if (b->slots[k].state == 1) {
      ++running;
      chunks += b->tab[k].chunks;
      tiles += (b->tab[k].ncell + b->tile_cells - 1) / b->tile_cells;
      const Params& q = b->tab[k].p;
      if (q.g.ndim != 2 || q.seg_alpha || q.limiter || q.quad) fused = false;
      else items += stage32_items(q);
    }
  }
  b->prefix[n] = chunks;
  b->tprefix[n] = tiles;
  b->s32prefix[n] = items;
  b->fast = fused;
  BCU(b, cudaMemcpyAsync(b->d_s32prefix, b->s32prefix.data(), (n + 1) * sizeof(long long),
                         cudaMemcpyHostToDevice, b->stream));
  BCU(b, cudaMemcpyAsync(b->d_prefix, b->prefix.data(), (n + 1) * sizeof(long long),
                         cudaMemcpyHostToDevice, b->stream));
  BCU(b, cudaMemcpyAsync(b->d_tprefix, b->tprefix.data(), (n + 1) * sizeof(long long),
                         cudaMemcpyHostToDevice, b->stream));
  BatchCtl& c = *b->h_ctl;
  c = BatchCtl{};
  c.n_active = running;
  c.total_chunks = chunks;
  c.total_tiles = tiles;
  c.tile_cells = b->tile_cells;
  c.steps_limit = max_steps;
  c.total_s32 = items;
  BCU(b, cudaMemcpyAsync(b->d_ctl, &c, sizeof(BatchCtl), cudaMemcpyHostToDevice, b->stream));
  return SWFD_OK;
}
}  // namespace

// cell-tile sizes the batch autotuner times, on findalpha over the running
// instances (it reads the state and writes only per-stage scratch)
swfd_status swfd_batch_autotune(swfd_batch* b, int32_t* tile_cells) {
  if (!b || !tile_cells) return bfail(b, SWFD_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(b->mu);
  BCU(b, cudaSetDevice(b->cfg.device));
  *tile_cells = b->tile_cells;
  int running = 0;
  for (const SlotHost& sh : b->slots) running += sh.state == 1;
  if (!running) return SWFD_OK;
  static const int cand[] = {512, 1024, 2048, 4096, 8192};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BCU(b, cudaEventCreate(&e0));
  BCU(b, cudaEventCreate(&e1));
  const BatchLaunch L = launch_desc(b);
  float best = 0.f;
  int pick = b->tile_cells;
  swfd_status st = SWFD_OK;
  for (int k = 0; k < (int)(sizeof(cand) / sizeof(cand[0])) && st == SWFD_OK; ++k) {
    b->tile_cells = cand[k];
    if ((st = upload_plan(b, 1)) != SWFD_OK) break;
    cudaError_t e = launch_batch_alpha(L, 0, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
    for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch_batch_alpha(L, 0, b->stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) {
      st = bfail(b, SWFD_ERR_CUDA, cudaGetErrorString(e));
      break;
    }
    if (k == 0 || ms < best) best = ms, pick = cand[k];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->tile_cells = pick;
  *tile_cells = pick;
  return st;
}

swfd_status swfd_batch_run(swfd_batch* b, int64_t max_steps, int64_t* steps_out) {
  if (!b) return bfail(b, SWFD_ERR_INVALID, "NULL handle");
  std::lock_guard<std::mutex> lk(b->mu);
  if (steps_out) *steps_out = 0;
  if (max_steps < 1) return bfail(b, SWFD_ERR_INVALID, "max_steps must be >= 1");
  BCU(b, cudaSetDevice(b->cfg.device));
  const int n = b->cfg.max_slots;
  int running = 0;
  for (int k = 0; k < n; ++k)
    if (b->slots[k].state == 1) {
      ++running;
      swfd_status st = ensure_slot_tracks(b, k, 3 * max_steps);
      if (st != SWFD_OK) return st;
    }
  if (!running) return SWFD_OK;
  {
    swfd_status st = upload_plan(b, max_steps);
    if (st != SWFD_OK) return st;
  }
  BCU(b, cudaGraphLaunch(b->fast ? b->g_fast : b->g_run, b->stream));
  BCU(b, cudaMemcpyAsync(b->h_ctl, b->d_ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, b->stream));
  BCU(b, cudaMemcpyAsync(b->tab.data(), b->d_tab, n * sizeof(BatchSlot), cudaMemcpyDeviceToHost,
                         b->stream));
  BCU(b, cudaMemcpyAsync(b->h_dsc, b->d_dsc, n * sizeof(DevScalars), cudaMemcpyDeviceToHost,
                         b->stream));
  BCU(b, cudaStreamSynchronize(b->stream));
  for (int k = 0; k < n; ++k) {
    SlotHost& sh = b->slots[k];
    if (sh.state != 1) continue;
    sh.last = b->h_dsc[k];
    if (!b->tab[k].active) {
      sh.state = 2;
      sh.status = status_of(sh.last.error);
    }
  }
  if (steps_out) *steps_out = b->h_ctl->steps;
  return SWFD_OK;
}

swfd_status swfd_batch_poll(swfd_batch* b, int64_t* ids, int32_t* status, int32_t cap,
                            int32_t* n_out) {
  if (!b || !n_out) return bfail(b, SWFD_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(b->mu);
  int32_t m = 0;
  for (auto& sh : b->slots) {
    if (sh.state != 2) continue;
    if (m >= cap) break;
    if (ids) ids[m] = sh.id;
    if (status) status[m] = sh.status;
    sh.state = 3;
    ++m;
  }
  *n_out = m;
  return SWFD_OK;
}

swfd_status swfd_batch_download(swfd_batch* b, int64_t request_id, double* u, double* time_out) {
  if (!b) return bfail(b, SWFD_ERR_INVALID, "NULL handle");
  std::lock_guard<std::mutex> lk(b->mu);
  int k = find_slot(b, request_id);
  if (k < 0) return bfail(b, SWFD_ERR_INVALID, "unknown request id");
  SlotHost& sh = b->slots[k];
  BCU(b, cudaSetDevice(b->cfg.device));
  if (u) {
    const size_t bytes = (size_t)sh.p.g.nc * sh.p.g.LI * sh.p.g.LJ * sizeof(double);
    BCU(b, launch_soa_to_fortran(sh.p, b->tab[k].st[0], b->d_stage, b->stream));
    BCU(b, cudaMemcpyAsync(u, b->d_stage, bytes, cudaMemcpyDeviceToHost, b->stream));
  }
  BCU(b, cudaMemcpyAsync(&sh.last, sh.dsc, sizeof(DevScalars), cudaMemcpyDeviceToHost, b->stream));
  BCU(b, cudaStreamSynchronize(b->stream));
  if (time_out) *time_out = sh.last.time;
  return SWFD_OK;
}

swfd_status swfd_batch_stats(swfd_batch* b, int64_t request_id, swfd_sweep_stats* s) {
  if (!b || !s) return bfail(b, SWFD_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(b->mu);
  int k = find_slot(b, request_id);
  if (k < 0) return bfail(b, SWFD_ERR_INVALID, "unknown request id");
  SlotHost& sh = b->slots[k];
  BCU(b, cudaSetDevice(b->cfg.device));
  BCU(b, cudaMemcpy(&sh.last, sh.dsc, sizeof(DevScalars), cudaMemcpyDeviceToHost));
  int64_t n = std::min<int64_t>(sh.last.sweep_count, sh.track_cap);
  std::vector<int32_t> tr(3 * (size_t)std::max<int64_t>(n, 1));
  for (int c = 0; c < 3 && n > 0; ++c)
    BCU(b, cudaMemcpy(tr.data() + c * n, sh.tracks + c * sh.track_cap, n * sizeof(int32_t),
                      cudaMemcpyDeviceToHost));
  memset(s, 0, sizeof(*s));
  s->sweep_count = sh.last.sweep_count;
  for (int64_t k2 = 0; k2 < n; ++k2) {
    int32_t sw = tr[k2], ng = tr[n + k2], ps = tr[2 * n + k2];
    s->total_sweep += sw;
    s->total_neg += ng;
    s->total_pos += ps;
    if (k2 == 0 || sw > s->max_sweep) s->max_sweep = sw;
    if (k2 == 0 || ng > s->max_neg) s->max_neg = ng;
    if (k2 == 0 || ps > s->max_pos) s->max_pos = ps;
  }
  s->den_count = sh.last.den_count;
  s->pre_count = sh.last.pre_count;
  s->sweep_fail_count = sh.last.fail_count;
  return SWFD_OK;
}

swfd_status swfd_batch_release(swfd_batch* b, int64_t request_id) {
  if (!b) return bfail(b, SWFD_ERR_INVALID, "NULL handle");
  std::lock_guard<std::mutex> lk(b->mu);
  int k = find_slot(b, request_id);
  if (k < 0) return bfail(b, SWFD_ERR_INVALID, "unknown request id");
  BCU(b, cudaSetDevice(b->cfg.device));
  swfd_status st = free_slot(b, k);
  BCU(b, cudaStreamSynchronize(b->stream));
  return st;
}

swfd_status swfd_batch_info(swfd_batch* b, int32_t* running, int32_t* free_slots,
                            int64_t* free_bytes) {
  if (!b) return bfail(b, SWFD_ERR_INVALID, "NULL handle");
  std::lock_guard<std::mutex> lk(b->mu);
  int32_t r = 0, f = 0;
  for (auto& sh : b->slots) {
    if (sh.state == 1) ++r;
    if (sh.state == 0) ++f;
  }
  if (running) *running = r;
  if (free_slots) *free_slots = f;
  if (free_bytes) *free_bytes = b->pool_bytes - b->used_bytes;
  return SWFD_OK;
}

swfd_status swfd_batch_progress(swfd_batch* b, int64_t request_id, double* time_out,
                                int64_t* steps_out) {
  if (!b) return bfail(b, SWFD_ERR_INVALID, "NULL handle");
  std::lock_guard<std::mutex> lk(b->mu);
  int k = find_slot(b, request_id);
  if (k < 0) return bfail(b, SWFD_ERR_INVALID, "unknown request id");
  const SlotHost& sh = b->slots[k];
  if (time_out) *time_out = sh.last.time;
  if (steps_out) *steps_out = sh.last.steps;
  return SWFD_OK;
}

swfd_status swfd_batch_get_stream(swfd_batch* b, void** stream) {
  if (!b || !stream) return bfail(b, SWFD_ERR_INVALID, "NULL argument");
  *stream = (void*)b->stream;
  return SWFD_OK;
}

}  // extern "C"
