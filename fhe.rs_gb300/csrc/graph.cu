// CUDA graphs of the batched multiplication and of the ragged rotation batch.
// The multiplication: the whole pipeline of
// Multiplicator::multiply for fixed device buffers recorded once and replayed
// with one launch call. A batch of 32 pairs or more is recorded as two
// branches of half the batch, each with its own scratch: running them side by
// side overlaps one branch's barriers, tails and latency-bound NTT phases with
// the other's multiplier-bound work (64 pairs at N = 2^14 on GB300: 2.55 ms
// as two concurrent halves against 2.62 ms as one batch).

#include <vector>

#include "abi_call.hpp"
#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

struct fheg_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  fheg::Workspace ws;    // scratch owned by the graph (never reallocated)
  fheg::Workspace ws2;   // scratch of the second branch
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

// Kernel nodes of a graph (counted into the launch counter per replay).
uint64_t kernel_nodes(cudaGraph_t graph) {
  size_t n = 0;
  fheg::check_cuda(cudaGraphGetNodes(graph, nullptr, &n), "cudaGraphGetNodes");
  std::vector<cudaGraphNode_t> nodes(n);
  if (n) fheg::check_cuda(cudaGraphGetNodes(graph, nodes.data(), &n), "cudaGraphGetNodes");
  uint64_t k = 0;
  for (cudaGraphNode_t node : nodes) {
    cudaGraphNodeType t;
    fheg::check_cuda(cudaGraphNodeGetType(node, &t), "cudaGraphNodeGetType");
    if (t == cudaGraphNodeTypeKernel) k++;
  }
  return k;
}

}  // namespace

FHEG_API int fheg_multiplicator_capture(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                        uint64_t* d_out, size_t count, fheg_graph** out) {
  fheg::set_last_error("");
  if (!m || !d_lhs || !d_rhs || !d_out || !count || !out)
    return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null input"));
  if (count > fheg::kMaxItems) return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "item count above 2^24 per call"));
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  auto release = [&] {
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  };
  auto g = new fheg_graph();
  try {
    fheg::Multiplicator& mult = *m->m;
    fheg::check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    fheg::check_cuda(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "cudaStreamCreate");
    fheg::check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    fheg::check_cuda(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "cudaEventCreate");
    // Branch 0 takes pairs [0, c0), branch 1 [c0, count).
    const size_t c0 = count >= 32 ? count / 2 : count;
    const size_t in_pair = 2 * mult.base->L() * mult.base->N();
    const size_t out_pair = mult.out_parts() * (mult.mod_switch ? mult.base->L() - 1 : mult.base->L()) *
                            mult.base->N();
    auto record = [&] {
      mult.multiply(d_lhs, d_rhs, d_out, c0, st, &g->ws);
      if (c0 < count)
        mult.multiply(d_lhs + c0 * in_pair, d_rhs + c0 * in_pair, d_out + c0 * out_pair, count - c0, st2, &g->ws2);
    };
    g->ws.reserve(mult.scratch_bytes(c0));
    if (c0 < count) g->ws2.reserve(mult.scratch_bytes(count - c0));
    // One ordinary run first: it sets every kernel attribute the pipeline
    // needs (a function attribute is not a stream operation) and checks the
    // arguments, so the capture below only records launches.
    record();
    fheg::check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    fheg::check_cuda(cudaStreamSynchronize(st2), "cudaStreamSynchronize");
    fheg::check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
      // st2 joins the capture by waiting on an event recorded in it, and
      // rejoins st before the capture ends.
      fheg::check_cuda(cudaEventRecord(fork, st), "cudaEventRecord");
      fheg::check_cuda(cudaStreamWaitEvent(st2, fork, 0), "cudaStreamWaitEvent");
      record();
      fheg::check_cuda(cudaEventRecord(join, st2), "cudaEventRecord");
      fheg::check_cuda(cudaStreamWaitEvent(st, join, 0), "cudaStreamWaitEvent");
    } catch (...) {
      cudaGraph_t partial = nullptr;
      cudaStreamEndCapture(st, &partial);
      if (partial) cudaGraphDestroy(partial);
      throw;
    }
    fheg::check_cuda(cudaStreamEndCapture(st, &g->graph), "cudaStreamEndCapture");
    fheg::check_cuda(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
    g->kernels = kernel_nodes(g->graph);
    release();
    *out = g;
    return FHEG_OK;
  } catch (const fheg::Error& e) {
    release();
    delete g;
    return fail(e);
  } catch (const std::exception& e) {
    release();
    delete g;
    return fail(fheg::Error(FHEG_ERR_INTERNAL, e.what()));
  }
}

FHEG_API int fheg_galois_relinearize_batch_capture(const fheg_params* par, const fheg_ksk* const* keys,
                                                   const size_t* exponents, const uint64_t* const* d_cts,
                                                   uint64_t* const* d_outs, size_t count, fheg_graph** out) {
  fheg::set_last_error("");
  if (!par || !out || !count || !keys || !exponents || !d_cts || !d_outs)
    return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null input"));
  if (count > fheg::kMaxItems) return fail(fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "item count above 2^24 per call"));
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  auto release = [&] {
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (st2) cudaStreamDestroy(st2);
    if (st) cudaStreamDestroy(st);
  };
  auto g = new fheg_graph();
  try {
    std::vector<fheg::RotRequest> req(count);
    for (size_t b = 0; b < count; b++) {
      if (!keys[b] || !d_cts[b] || !d_outs[b] || d_cts[b] == d_outs[b])
        throw fheg::Error(FHEG_ERR_INVALID_ARGUMENT, "null or aliased batch entry");
      req[b] = fheg::RotRequest{&keys[b]->k, exponents[b], d_cts[b], d_outs[b]};
    }
    const fheg::Params& p = *par->p;
    fheg::validate_rot_requests(p, req.data(), count);
    fheg::check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    fheg::check_cuda(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking), "cudaStreamCreate");
    fheg::check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    fheg::check_cuda(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "cudaEventCreate");
    // As the direct call: from 16 requests two halves side by side, each
    // with its tables and scratch in the graph's own workspaces.
    const size_t c0 = count >= 16 ? count / 2 : count;
    auto run0 = fheg::prepare_galois_batch(p, req.data(), c0, g->ws, st);
    auto run1 = fheg::prepare_galois_batch(p, req.data() + c0, count - c0, g->ws2, st);
    // One ordinary run sets every kernel attribute before the capture.
    run0(st);
    run1(st2);
    fheg::check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    fheg::check_cuda(cudaStreamSynchronize(st2), "cudaStreamSynchronize");
    fheg::check_cuda(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    try {
      fheg::check_cuda(cudaEventRecord(fork, st), "cudaEventRecord");
      fheg::check_cuda(cudaStreamWaitEvent(st2, fork, 0), "cudaStreamWaitEvent");
      run0(st);
      run1(st2);
      fheg::check_cuda(cudaEventRecord(join, st2), "cudaEventRecord");
      fheg::check_cuda(cudaStreamWaitEvent(st, join, 0), "cudaStreamWaitEvent");
    } catch (...) {
      cudaGraph_t partial = nullptr;
      cudaStreamEndCapture(st, &partial);
      if (partial) cudaGraphDestroy(partial);
      throw;
    }
    fheg::check_cuda(cudaStreamEndCapture(st, &g->graph), "cudaStreamEndCapture");
    fheg::check_cuda(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
    g->kernels = kernel_nodes(g->graph);
    release();
    *out = g;
    return FHEG_OK;
  } catch (const fheg::Error& e) {
    release();
    delete g;
    return fail(e);
  } catch (const std::exception& e) {
    release();
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
