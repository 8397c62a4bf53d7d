// swfd_graph.h -- building CUDA graphs with device-side conditional nodes.
#pragma once

#include <string.h>

#include "swfd_internal.h"

namespace swfd {

// ---------------------------------------------------------------------------
// Graph construction.  Work is recorded by stream capture; a conditional node
// is spliced into the capture (cudaStreamGetCaptureInfo + cudaGraphAddNode +
// cudaStreamUpdateCaptureDependencies) and its body is captured on the
// stream of the next nesting depth.  The control kernels of swfd_control.cu
// set the conditions on the device.
//
// In eager mode the same emitters launch directly on the stream: handles are
// 0, the control kernels write each decision to a condition word, and cond()
// reads it back (after a stream synchronisation) to run a body once (IF) or
// while it stays set (WHILE).
// ---------------------------------------------------------------------------
struct Builder {
  swfd_handle* h = nullptr;
  cudaStream_t* cap = nullptr;  // capture streams, one per nesting depth
  int max_depth = 0;            // capture streams available beyond depth 0
  cudaGraph_t root = nullptr;
  int depth = 0;
  int* count = nullptr;  // kernels emitted into the current section
  cudaError_t err = cudaSuccess;
  bool eager = false;
  const int* cond_word = nullptr;  // eager: device word the control kernels write
  long long* launched = nullptr;   // eager: kernels launched
  bool ok(cudaError_t e) {
    if (e != cudaSuccess && err == cudaSuccess) err = e;
    return err == cudaSuccess;
  }
  void k(int n) {
    if (count) *count += n;
    if (launched) *launched += n;
  }
  bool read_cond(cudaStream_t s) {
    int v = 0;
    if (!ok(cudaStreamSynchronize(s))) return false;
    if (!ok(cudaMemcpy(&v, cond_word, sizeof(int), cudaMemcpyDeviceToHost))) return false;
    return v != 0;
  }
  template <class F>
  void cond(cudaStream_t s, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle hnd,
            F body) {
    if (err != cudaSuccess) return;
    if (eager) {
      if (type == cudaGraphCondTypeIf) {
        if (read_cond(s)) body(s);
      } else {
        while (err == cudaSuccess && read_cond(s)) body(s);
      }
      return;
    }
    if (depth + 1 > max_depth) {
      err = cudaErrorInvalidValue;
      return;
    }
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    if (!ok(cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd))) return;
    // cudaGraphNodeParams has no default constructor (its union holds
    // members with constructors): build it in zeroed raw storage
    alignas(cudaGraphNodeParams) unsigned char raw[sizeof(cudaGraphNodeParams)];
    memset(raw, 0, sizeof(raw));
    cudaGraphNodeParams* np = reinterpret_cast<cudaGraphNodeParams*>(raw);
    np->type = cudaGraphNodeTypeConditional;
    np->conditional.handle = hnd;
    np->conditional.type = type;
    np->conditional.size = 1;
    cudaGraphNode_t node;
    if (!ok(cudaGraphAddNode(&node, g, deps, nullptr, nd, np))) return;
    if (!ok(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1,
                                                cudaStreamSetCaptureDependencies)))
      return;
    cudaGraph_t bg = np->conditional.phGraph_out[0];
    cudaStream_t sb = cap[++depth];
    if (ok(cudaStreamBeginCaptureToGraph(sb, bg, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeRelaxed))) {
      body(sb);
      cudaGraph_t tmp;
      ok(cudaStreamEndCapture(sb, &tmp));
    }
    --depth;
  }
  cudaGraphConditionalHandle handle() {
    cudaGraphConditionalHandle hnd = 0;
    if (eager) return 0;
    ok(cudaGraphConditionalHandleCreate(&hnd, root, 0, 0));
    // handle 0 selects the eager path in the control kernels
    if (err == cudaSuccess && hnd == 0) err = cudaErrorUnknown;
    return hnd;
  }
};

#define B_OK(b, call) \
  do {                \
    (b).ok(call);     \
  } while (0)


}  // namespace swfd
