// swfd_static.cu -- swfd_flux_divergence_static: the flux divergence
// (wenofd + scheme) of a state the caller already holds on the device, with
// every intermediate array in one file-scope device array instead of memory
// allocated per call or per handle.
//
// It is for callers that cannot call cudaMalloc: code running under an
// allocator that owns all device memory (a framework's caching allocator or a
// memory pool that forbids outside allocations), real-time loops where an
// allocation could block, and callers that only hand over device pointers
// they were given.  The caller passes the input state and the output array;
// the library allocates nothing.
//
// Limits and sharing:
//  - the scratch array is SWFD_STATIC_SCRATCH_BYTES (8 MiB) of device memory
//    that every GPU which loads this library keeps until the process exits;
//    grids whose intermediates do not fit are rejected with SWFD_ERR_INVALID
//    (in 2D about 130 x 130 interior cells; in 1D about 27000 cells);
//  - all calls share the one array and it keeps the previous call's contents,
//    so the entry point clears what must start at zero on every call;
//  - two calls whose work overlaps on the GPU (different streams, or
//    different host threads on the same device without ordering) race on the
//    array and corrupt each other's results: order them on one stream;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture begins.  Later calls on a stream that is not
//    capturing look it up again, so a context torn down by cudaDeviceReset
//    and created anew is followed; a call made while the stream captures
//    uses the address of the last call outside capture.
#include <mutex>
#include <string>

#include "swfd_internal.h"

#define SWFD_STATIC_SCRATCH_BYTES (8u << 20)
#define SWFD_STATIC_MAX_DEVICES 64

namespace {

// The scratch itself.  In host code this name is only a host-side stand-in
// for the device array, never a device address: the address is looked up with
// cudaGetSymbolAddress and cached per device.
static __device__ __align__(256) unsigned char g_static_scratch[SWFD_STATIC_SCRATCH_BYTES];

std::mutex g_static_mu;
void* g_static_addr[SWFD_STATIC_MAX_DEVICES] = {nullptr};

swfd_status static_fail(swfd_status st, const std::string& m) {
  swfd::set_last_error(m);  // readable with swfd_last_error(NULL, ...)
  return st;
}

// device address of g_static_scratch on `dev` (dev must be current).  Outside
// stream capture the address is looked up every time (a cudaDeviceReset
// unloads the module, and the next context may place the array elsewhere);
// during capture the address of the last lookup is used, and a first call on
// a device made during capture is refused.
cudaError_t static_scratch_addr(int dev, cudaStream_t s, void** out) {
  std::lock_guard<std::mutex> lk(g_static_mu);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  const bool capturing = cudaStreamIsCapturing(s, &cs) != cudaSuccess ||
                         cs != cudaStreamCaptureStatusNone;
  if (capturing) {
    cudaGetLastError();  // a refused capture query leaves no sticky error
    if (!g_static_addr[dev]) return cudaErrorStreamCaptureUnsupported;
  } else {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return cudaSuccess;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" swfd_status swfd_flux_divergence_static(const swfd_config* cfg, const double* u,
                                                   double* rhs, void* stream) {
  using namespace swfd;
  if (!cfg || !u || !rhs) return static_fail(SWFD_ERR_INVALID, "NULL argument");
  std::string err;
  swfd_status st = check_config(*cfg, err);
  if (st != SWFD_OK) return static_fail(st, err);
  if (cfg->problem == SWFD_PROBLEM_DETONATION)
    return static_fail(SWFD_ERR_UNSUPPORTED, "the detonation needs per-rank buffers: use swfd_step");
  Params p;
  st = make_params(*cfg, p, err);
  if (st != SWFD_OK) return static_fail(st, err);
  if (p.quad)
    return static_fail(SWFD_ERR_UNSUPPORTED, "swfd_flux_divergence_static: binary64 literals only");
  if (p.problem == SWFD_PROBLEM_MATLAB_1D)
    return static_fail(SWFD_ERR_UNSUPPORTED, "the MATLAB script's scheme runs whole steps only");
  if (p.seg_alpha)
    return static_fail(SWFD_ERR_UNSUPPORTED,
                       "shock diffraction needs per-rank buffers: use swfd_flux_divergence");
  const Geom& g = p.g;
  // intermediates: SoA state (nc planes), split fluxes (4 nc), Roe averages
  // (8), interface fluxes (4 nc), SoA RHS (nc), device scalars
  const size_t plane_b = align256((size_t)g.plane * sizeof(double));
  const size_t need = (size_t)(10 * g.nc + 8) * plane_b + align256(sizeof(DevScalars));
  if (need > SWFD_STATIC_SCRATCH_BYTES)
    return static_fail(SWFD_ERR_INVALID,
                       "grid too large for swfd_flux_divergence_static: needs " +
                           std::to_string(need) + " bytes of scratch, the static limit is " +
                           std::to_string(SWFD_STATIC_SCRATCH_BYTES) + " bytes");
  if (cfg->device < 0 || cfg->device >= SWFD_STATIC_MAX_DEVICES)
    return static_fail(SWFD_ERR_INVALID, "device ordinal out of range");
  int prev = -1;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) return static_fail(SWFD_ERR_CUDA, cudaGetErrorString(e));
  if (prev != cfg->device && (e = cudaSetDevice(cfg->device)) != cudaSuccess)
    return static_fail(SWFD_ERR_CUDA, cudaGetErrorString(e));
  auto done = [&](swfd_status s, const char* what, cudaError_t ce) -> swfd_status {
    if (prev != cfg->device) cudaSetDevice(prev);
    if (s != SWFD_OK) return static_fail(s, std::string(what) + ": " + cudaGetErrorString(ce));
    return SWFD_OK;
  };
  cudaStream_t s = (cudaStream_t)stream;
  void* base = nullptr;
  if ((e = static_scratch_addr(cfg->device, s, &base)) != cudaSuccess)
    return done(SWFD_ERR_CUDA, "cudaGetSymbolAddress", e);
  char* c = (char*)base;
  DevScalars* dsc = (DevScalars*)c;
  c += align256(sizeof(DevScalars));
  double* usoa = (double*)c;
  c += g.nc * plane_b;
  double* split = (double*)c;
  c += 4 * g.nc * plane_b;
  double* roe = (double*)c;
  c += 8 * plane_b;
  double* flux = (double*)c;
  c += 4 * g.nc * plane_b;
  double* rsoa = (double*)c;
  // the plane pitch used by the kernels must match the carved planes; the
  // split and flux planes (geometry sg) equal the state's here (problems with
  // rank segments are refused above)
  Params q = p;
  q.g.plane = (int64_t)(plane_b / sizeof(double));
  q.sg = q.g;
  // the previous call's scalars (alpha accumulator, error word) start at zero
  if ((e = cudaMemsetAsync(dsc, 0, sizeof(DevScalars), s)) != cudaSuccess)
    return done(SWFD_ERR_CUDA, "cudaMemsetAsync", e);
  if ((e = launch_fortran_to_soa(q, u, usoa, s)) != cudaSuccess ||
      (e = launch_alpha(q, usoa, dsc, s)) != cudaSuccess ||
      (e = launch_prep(q, usoa, dsc, split, roe, s)) != cudaSuccess ||
      (e = launch_flux(q, split, g.ndim == 1 ? usoa : roe, dsc, flux, &dsc->flux_work, s)) != cudaSuccess ||
      (e = launch_rhs(q, flux, dsc, rsoa, s)) != cudaSuccess ||
      (e = launch_soa_to_fortran(q, rsoa, rhs, s)) != cudaSuccess)
    return done(SWFD_ERR_CUDA, "kernel launch", e);
  return done(SWFD_OK, "", cudaSuccess);
}
