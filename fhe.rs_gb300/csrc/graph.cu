// CUDA graphs of the batched multiplication: the whole pipeline of
// Multiplicator::multiply for fixed device buffers recorded once and replayed
// with one launch call.

#include <vector>

#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

struct fheg_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  fheg::Workspace ws;    // scratch owned by the graph (never reallocated)
  uint64_t kernels = 0;  // kernel nodes, counted into the launch counter per replay
  ~fheg_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

namespace {

int fail(const fheg::Error& e) {
  fheg::set_last_error(e.what());
  return e.code;
}

}  // namespace

FHEG_API int fheg_multiplicator_capture(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                        uint64_t* d_out, size_t count, fheg_graph** out) {
  fheg::set_last_error("");
  if (!m || !d_lhs || !d_rhs || !d_out || !count || !out)
    return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null input"));
  cudaStream_t st = nullptr;
  auto g = new fheg_graph();
  try {
    fheg::Multiplicator& mult = *m->m;
    fheg::check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    g->ws.reserve(mult.scratch_bytes(count));
    // One ordinary run first: it sets every kernel attribute the pipeline
    // needs (a function attribute is not a stream operation) and checks the
    // arguments, so the capture below only records launches.
    mult.multiply(d_lhs, d_rhs, d_out, count, st, &g->ws);
    fheg::check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    fheg::check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
      mult.multiply(d_lhs, d_rhs, d_out, count, st, &g->ws);
    } catch (...) {
      cudaGraph_t partial = nullptr;
      cudaStreamEndCapture(st, &partial);
      if (partial) cudaGraphDestroy(partial);
      throw;
    }
    fheg::check_cuda(cudaStreamEndCapture(st, &g->graph), "cudaStreamEndCapture");
    fheg::check_cuda(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
    size_t n = 0;
    fheg::check_cuda(cudaGraphGetNodes(g->graph, nullptr, &n), "cudaGraphGetNodes");
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) fheg::check_cuda(cudaGraphGetNodes(g->graph, nodes.data(), &n), "cudaGraphGetNodes");
    for (cudaGraphNode_t node : nodes) {
      cudaGraphNodeType t;
      fheg::check_cuda(cudaGraphNodeGetType(node, &t), "cudaGraphNodeGetType");
      if (t == cudaGraphNodeTypeKernel) g->kernels++;
    }
    cudaStreamDestroy(st);
    *out = g;
    return FHEG_OK;
  } catch (const fheg::Error& e) {
    if (st) cudaStreamDestroy(st);
    delete g;
    return fail(e);
  } catch (const std::exception& e) {
    if (st) cudaStreamDestroy(st);
    delete g;
    return fail(fheg::Error(FHEG_ERR_INTERNAL, e.what()));
  }
}

FHEG_API int fheg_graph_launch(const fheg_graph* g, void* stream) {
  fheg::set_last_error("");
  if (!g) return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null graph"));
  const cudaError_t e = cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return fail(fheg::Error(FHEG_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e)));
  fheg::g_launches.fetch_add(g->kernels, std::memory_order_relaxed);
  return FHEG_OK;
}

FHEG_API int fheg_graph_kernel_count(const fheg_graph* g, uint64_t* kernels) {
  if (!g || !kernels) return FHEG_ERR_INVALID_ARGUMENT;
  *kernels = g->kernels;
  return FHEG_OK;
}

FHEG_API void fheg_graph_destroy(fheg_graph* g) { delete g; }
