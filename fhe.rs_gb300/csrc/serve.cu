// Serving runtime: continuous batching of mixed BFV requests on one GPU.
//
// Requests (mul+relin, rotation, addition, switch-down) are submitted from
// any thread with host buffers. A scheduler thread groups pending requests
// that can share a launch (same operation and parameters; rotations with
// different keys and levels batch together through the ragged path), admits a
// batch when a stream slot is free and its device memory (inputs, outputs and
// the operation's scratch) fits in the fixed HBM budget, copies the inputs,
// runs the batched operation and copies the outputs back, all on the slot's
// stream. Requests that arrive while others run are admitted as soon as a
// slot and memory free up, so copies and kernels of different batches overlap
// on the device. Completion is detected with CUDA events polled by the
// scheduler; host waits are bounded by a caller timeout.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <string>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

namespace {

using fheg::Error;

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// First-fit allocator over one device allocation (256-byte granules).
struct Arena {
  fheg::DevBuf mem;
  std::map<size_t, size_t> free_;  // offset -> bytes
  size_t used = 0, peak = 0;

  void init(size_t bytes) {
    mem.alloc(bytes);
    free_.clear();
    free_[0] = bytes;
  }
  static size_t round(size_t b) { return (b + 255) & ~(size_t)255; }
  bool alloc(size_t bytes, size_t* off) {
    bytes = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t noff = it->first + bytes;
        free_.erase(it);
        if (rest) free_[noff] = rest;
        used += bytes;
        peak = std::max(peak, used);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = round(bytes);
    used -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_.erase(next);
    }
    if (it != free_.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_.erase(it);
      }
    }
  }
  uint8_t* base() const { return static_cast<uint8_t*>(mem.ptr); }
};

struct Req {
  fheg_request r;
  uint64_t id;
  int status = -1;  // -1 while pending or running
  std::string err;
  int64_t t_submit = 0, t_start = 0, t_done = 0;
  size_t in_words = 0, out_words = 0;  // per operand / output
  size_t L = 0, out_L = 0, out_parts = 0, N = 0;
  uint64_t group = 0;  // requests with equal groups can share a launch
};

// Pinned host staging for requests whose host buffers are pageable: inputs
// are copied into it before their upload, outputs land in it and are copied
// to the caller's buffer when the batch completes.
struct Staging {
  uint64_t* ptr = nullptr;
  size_t words = 0;
  Staging() {}
  Staging(const Staging&) = delete;
  Staging& operator=(const Staging&) = delete;
  Staging(Staging&& o) noexcept : ptr(o.ptr), words(o.words) {
    o.ptr = nullptr;
    o.words = 0;
  }
  void reserve(size_t w) {
    if (w <= words) return;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    words = 0;
    fheg::check_cuda(cudaHostAlloc(reinterpret_cast<void**>(&ptr), w * 8, cudaHostAllocDefault), "cudaHostAlloc");
    words = w;
  }
  ~Staging() {
    if (ptr) cudaFreeHost(ptr);
  }
};

struct CopyBack {
  uint64_t* dst;
  size_t stage_off, words;
};

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  bool busy = false;
  std::vector<uint64_t> ids;
  size_t off = 0, bytes = 0;
  Staging stage;
  std::vector<CopyBack> copy_back;
};

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

}  // namespace

struct fheg_server {
  fheg_server_config cfg;
  Arena arena;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> pending;
  std::unordered_map<uint64_t, Req> reqs;  // element references stay valid across inserts
  uint64_t next_id = 1;
  uint64_t submitted = 0, completed = 0, batches = 0;
  bool stop = false;
  int device = 0;
  std::thread worker;

  void run();
  bool pick(Slot& s, std::vector<Req*>& batch, size_t* scratch);
  void launch(Slot& s, const std::vector<Req*>& batch, size_t scratch);
  void retire(Slot& s);
  void fail(Slot& s, int code, const std::string& msg);
};

namespace {

// Sizes and grouping key of a request; throws on an invalid request.
void describe(Req& q) {
  const fheg_request& r = q.r;
  if (!r.par || !r.in0 || !r.out) throw Error(FHEG_ERR_INVALID_ARGUMENT, "request without parameters or buffers");
  const fheg::Params& par = *r.par->p;
  q.N = par.degree;
  switch (r.op) {
    case FHEG_OP_MUL_RELIN: {
      if (!r.mult || !r.in1) throw Error(FHEG_ERR_INVALID_ARGUMENT, "mul+relin needs a multiplicator and two inputs");
      const fheg::Multiplicator& m = *r.mult->m;
      if (m.par != &par) throw Error(FHEG_ERR_KEY_MISMATCH, "multiplicator of other parameters");
      q.L = m.base->L();
      q.out_parts = m.out_parts();
      q.out_L = par.ctx(m.out_level())->L();
      // One group per parameter set: a batch may mix levels (multiplicators)
      // and runs as one sub-batch per multiplicator.
      q.group = (uint64_t)(uintptr_t)m.par * 8 + 0;
      break;
    }
    case FHEG_OP_ROTATE: {
      if (!r.key) throw Error(FHEG_ERR_INVALID_ARGUMENT, "rotation needs a Galois key");
      if (r.key->k.par != &par) throw Error(FHEG_ERR_KEY_MISMATCH, "key of other parameters");
      if ((r.exponent % (2 * q.N)) % 2 == 0)
        throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
      q.L = q.out_L = r.key->k.ctx_ct->L();
      q.out_parts = 2;
      q.group = (uint64_t)(uintptr_t)r.par * 8 + 1;
      break;
    }
    case FHEG_OP_ADD: {
      if (!r.in1) throw Error(FHEG_ERR_INVALID_ARGUMENT, "addition needs two inputs");
      q.L = q.out_L = par.ctx(r.level)->L();
      q.out_parts = 2;
      q.group = ((uint64_t)(uintptr_t)r.par * 8 + 2) ^ ((uint64_t)r.level << 48);
      break;
    }
    case FHEG_OP_SWITCH_DOWN: {
      if (r.level >= par.max_level()) throw Error(FHEG_ERR_NO_MORE_CONTEXT, "NoMoreContext");
      q.L = par.ctx(r.level)->L();
      q.out_L = q.L - 1;
      q.out_parts = 2;
      q.group = ((uint64_t)(uintptr_t)r.par * 8 + 3) ^ ((uint64_t)r.level << 48);
      break;
    }
    default:
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "unknown operation");
  }
  q.in_words = 2 * q.L * q.N;
  q.out_words = q.out_parts * q.out_L * q.N;
}

size_t batch_io_bytes(const std::vector<Req*>& b) {
  size_t words = 0;
  for (Req* q : b) words += (q->r.op == FHEG_OP_MUL_RELIN || q->r.op == FHEG_OP_ADD ? 2 : 1) * q->in_words + q->out_words;
  // Each carved region is rounded up to 256 bytes: at most four per request
  // (mul+relin sub-batches: inputs, output, scratch), plus a few.
  return words * 8 + (4 * b.size() + 4) * 256;
}

// The mul+relin requests of a batch split by multiplicator, in order of
// first appearance (each sub-batch keeps arrival order).
std::vector<std::vector<Req*>> by_multiplicator(const std::vector<Req*>& b) {
  std::vector<std::vector<Req*>> groups;
  for (Req* q : b) {
    size_t g = 0;
    while (g < groups.size() && groups[g][0]->r.mult != q->r.mult) g++;
    if (g == groups.size()) groups.emplace_back();
    groups[g].push_back(q);
  }
  return groups;
}

size_t batch_scratch_bytes(const std::vector<Req*>& b) {
  const Req& q = *b[0];
  switch (q.r.op) {
    case FHEG_OP_MUL_RELIN: {
      size_t bytes = 0;
      for (const auto& g : by_multiplicator(b)) bytes += g[0]->r.mult->m->scratch_bytes(g.size()) + 256;
      return bytes;
    }
    case FHEG_OP_ROTATE: {
      std::vector<fheg::RotRequest> rr;
      for (Req* x : b) rr.push_back(fheg::RotRequest{&x->r.key->k, x->r.exponent, nullptr, nullptr});
      return fheg::galois_batch_scratch_bytes(rr.data(), rr.size());
    }
    default:
      return 0;
  }
}

}  // namespace

void fheg_server::launch(Slot& s, const std::vector<Req*>& batch, size_t scratch_bytes) {
  const Req& q0 = *batch[0];
  const size_t B = batch.size();
  cudaStream_t st = s.stream;
  uint64_t* p = reinterpret_cast<uint64_t*>(arena.base() + s.off);
  auto carve = [&](size_t words) {
    uint64_t* r = p;
    p += (words + 31) & ~(size_t)31;
    return r;
  };
  // Host staging needed by pageable buffers of this batch.
  size_t stage_words = 0;
  std::vector<char> pin_in0(B), pin_in1(B), pin_out(B);
  for (size_t k = 0; k < B; k++) {
    const Req& q = *batch[k];
    pin_in0[k] = is_pinned(q.r.in0);
    pin_in1[k] = q.r.in1 ? is_pinned(q.r.in1) : 1;
    pin_out[k] = is_pinned(q.r.out);
    stage_words += (pin_in0[k] ? 0 : q.in_words) + (pin_in1[k] ? 0 : q.in_words) + (pin_out[k] ? 0 : q.out_words);
  }
  s.stage.reserve(stage_words);
  size_t stage_off = 0;
  s.copy_back.clear();
  auto h2d = [&](uint64_t* d, const uint64_t* h, size_t words, bool pinned) {
    if (!pinned) {
      uint64_t* t = s.stage.ptr + stage_off;
      std::memcpy(t, h, words * 8);
      stage_off += words;
      h = t;
    }
    fheg::check_cuda(cudaMemcpyAsync(d, h, words * 8, cudaMemcpyHostToDevice, st), "H2D");
  };
  auto d2h = [&](uint64_t* h, const uint64_t* d, size_t words, bool pinned) {
    if (!pinned) {
      s.copy_back.push_back(CopyBack{h, stage_off, words});
      h = s.stage.ptr + stage_off;
      stage_off += words;
    }
    fheg::check_cuda(cudaMemcpyAsync(h, d, words * 8, cudaMemcpyDeviceToHost, st), "D2H");
  };
  fheg::Workspace ws;
  if (q0.r.op == FHEG_OP_MUL_RELIN) {
    // One sub-batch per multiplicator (level), one after the other on the
    // slot's stream, each with its own inputs, outputs and scratch.
    for (const auto& g : by_multiplicator(batch)) {
      const Req& g0 = *g[0];
      const size_t G = g.size();
      uint64_t* a = carve(G * g0.in_words);
      uint64_t* b = carve(G * g0.in_words);
      uint64_t* o = carve(G * g0.out_words);
      for (size_t k = 0; k < G; k++) {
        const size_t i = (size_t)(std::find(batch.begin(), batch.end(), g[k]) - batch.begin());
        h2d(a + k * g0.in_words, g[k]->r.in0, g0.in_words, pin_in0[i]);
        h2d(b + k * g0.in_words, g[k]->r.in1, g0.in_words, pin_in1[i]);
      }
      const size_t sb = g0.r.mult->m->scratch_bytes(G);
      fheg::Workspace gws;
      gws.attach(carve(sb / 8), sb);
      g0.r.mult->m->multiply(a, b, o, G, st, &gws);
      for (size_t k = 0; k < G; k++) {
        const size_t i = (size_t)(std::find(batch.begin(), batch.end(), g[k]) - batch.begin());
        d2h(g[k]->r.out, o + k * g0.out_words, g0.out_words, pin_out[i]);
      }
    }
  } else if (q0.r.op == FHEG_OP_ADD) {
    uint64_t* a = carve(B * q0.in_words);
    uint64_t* b = carve(B * q0.in_words);
    uint64_t* o = carve(B * q0.out_words);
    for (size_t k = 0; k < B; k++) {
      h2d(a + k * q0.in_words, batch[k]->r.in0, q0.in_words, pin_in0[k]);
      h2d(b + k * q0.in_words, batch[k]->r.in1, q0.in_words, pin_in1[k]);
    }
    const fheg::Context& c = *q0.r.par->p->ctx(q0.r.level);
    fheg::PolyRef ra = fheg::plain_ref(a, c.L(), c.logn), rb = fheg::plain_ref(b, c.L(), c.logn),
                  ro = fheg::plain_ref(o, c.L(), c.logn);
    fheg::poly_op(c, 0, ra, rb, ro, 2 * B, st);
    for (size_t k = 0; k < B; k++) d2h(batch[k]->r.out, o + k * q0.out_words, q0.out_words, pin_out[k]);
  } else if (q0.r.op == FHEG_OP_SWITCH_DOWN) {
    uint64_t* a = carve(B * q0.in_words);
    uint64_t* o = carve(B * q0.out_words);
    for (size_t k = 0; k < B; k++) h2d(a + k * q0.in_words, batch[k]->r.in0, q0.in_words, pin_in0[k]);
    fheg::ciphertext_switch_down(*q0.r.par->p, q0.r.level, 2, a, o, B, st);
    for (size_t k = 0; k < B; k++) d2h(batch[k]->r.out, o + k * q0.out_words, q0.out_words, pin_out[k]);
  } else {  // rotations: one ragged launch sequence for any keys and levels
    std::vector<fheg::RotRequest> rr(B);
    for (size_t k = 0; k < B; k++) {
      Req& q = *batch[k];
      uint64_t* a = carve(q.in_words);
      uint64_t* o = carve(q.out_words);
      h2d(a, q.r.in0, q.in_words, pin_in0[k]);
      rr[k] = fheg::RotRequest{&q.r.key->k, q.r.exponent, a, o};
    }
    ws.attach(carve(scratch_bytes / 8), scratch_bytes);
    fheg::galois_relinearize_batch(*q0.r.par->p, rr.data(), B, ws, st);
    for (size_t k = 0; k < B; k++) d2h(batch[k]->r.out, rr[k].out, batch[k]->out_words, pin_out[k]);
  }
  fheg::check_cuda(cudaEventRecord(s.done, st), "cudaEventRecord");
}

// Chooses the next batch for a free slot (called with the lock held): the
// oldest pending request and the pending requests of its group, in arrival
// order, shrunk until inputs, outputs and scratch fit in the arena.
bool fheg_server::pick(Slot& s, std::vector<Req*>& batch, size_t* scratch) {
  batch.clear();
  if (pending.empty()) return false;
  const uint64_t g = reqs.at(pending.front()).group;
  for (uint64_t id : pending) {
    Req& q = reqs.at(id);
    if (q.group == g) batch.push_back(&q);
    if (batch.size() >= cfg.max_batch) break;
  }
  size_t off = 0, bytes = 0;
  while (!batch.empty()) {
    *scratch = batch_scratch_bytes(batch);
    bytes = batch_io_bytes(batch) + *scratch;
    if (arena.alloc(bytes, &off)) break;
    batch.pop_back();
  }
  if (batch.empty()) {
    const bool idle = std::none_of(slots.begin(), slots.end(), [](const Slot& x) { return x.busy; });
    if (idle) {  // the whole arena is free and the request still does not fit
      Req& q = reqs.at(pending.front());
      q.status = FHEG_ERR_BUDGET;
      q.err = "request exceeds the server's device memory budget";
      q.t_start = q.t_done = now_ns();
      pending.pop_front();
      completed++;
      cv_done.notify_all();
    }
    return false;
  }
  std::vector<uint64_t> ids;
  for (Req* q : batch) ids.push_back(q->id);
  size_t taken = 0;
  for (auto it = pending.begin(); it != pending.end() && taken < ids.size();) {
    if (std::find(ids.begin(), ids.end(), *it) != ids.end()) {
      it = pending.erase(it);
      taken++;
    } else {
      ++it;
    }
  }
  const int64_t t = now_ns();
  for (Req* q : batch) q->t_start = t;
  s.ids = std::move(ids);
  s.off = off;
  s.bytes = bytes;
  s.busy = true;
  batches++;
  return true;
}

void fheg_server::retire(Slot& s) {
  for (const CopyBack& c : s.copy_back) std::memcpy(c.dst, s.stage.ptr + c.stage_off, c.words * 8);
  s.copy_back.clear();
  const int64_t t = now_ns();
  for (uint64_t id : s.ids) {
    Req& q = reqs.at(id);
    if (q.status < 0) q.status = FHEG_OK;
    q.t_done = t;
    completed++;
  }
  arena.release(s.off, s.bytes);
  s.ids.clear();
  s.busy = false;
  cv_done.notify_all();
}

void fheg_server::fail(Slot& s, int code, const std::string& msg) {
  for (uint64_t id : s.ids) {
    Req& q = reqs.at(id);
    q.status = code;
    q.err = msg;
  }
  s.copy_back.clear();
}

void fheg_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lock(mu);
  std::vector<Req*> batch;
  for (;;) {
    for (Slot& s : slots) {
      if (!s.busy) continue;
      const cudaError_t e = cudaEventQuery(s.done);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) fail(s, FHEG_ERR_CUDA, cudaGetErrorString(e));
      retire(s);
    }
    for (Slot& s : slots) {
      if (s.busy) continue;
      size_t scratch = 0;
      if (!pick(s, batch, &scratch)) continue;
      // Enqueue without the lock so that submitters are not held up.
      lock.unlock();
      int code = FHEG_OK;
      std::string msg;
      try {
        launch(s, batch, scratch);
      } catch (const fheg::Error& e) {
        code = e.code;
        msg = e.what();
      } catch (const std::exception& e) {
        code = FHEG_ERR_INTERNAL;
        msg = e.what();
      }
      if (code != FHEG_OK) cudaStreamSynchronize(s.stream);  // issued copies end before the memory is reused
      lock.lock();
      if (code != FHEG_OK) {
        fail(s, code, msg);
        retire(s);
      }
    }
    const bool any_busy = std::any_of(slots.begin(), slots.end(), [](const Slot& x) { return x.busy; });
    if (stop && !any_busy && pending.empty()) break;
    // Poll the running batches' events every few microseconds; otherwise
    // sleep until a submission arrives.
    if (any_busy) cv_work.wait_for(lock, std::chrono::microseconds(20));
    else if (pending.empty()) cv_work.wait_for(lock, std::chrono::milliseconds(50));
  }
}

FHEG_API int fheg_server_create(const fheg_server_config* cfg, fheg_server** out) {
  try {
    fheg::set_last_error("");
    if (!cfg || !out || cfg->hbm_budget_bytes < (1u << 20) || cfg->streams == 0 || cfg->max_batch == 0)
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "invalid server configuration");
    auto s = new fheg_server();
    s->cfg = *cfg;
    try {
      fheg::check_cuda(cudaGetDevice(&s->device), "cudaGetDevice");
      s->arena.init(cfg->hbm_budget_bytes);
      s->slots.resize(cfg->streams);
      for (Slot& sl : s->slots) {
        fheg::check_cuda(cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking), "stream");
        fheg::check_cuda(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming), "event");
      }
      s->worker = std::thread([s] { s->run(); });
    } catch (...) {
      for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
      }
      delete s;
      throw;
    }
    *out = s;
    return FHEG_OK;
  } catch (const Error& e) {
    fheg::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    fheg::set_last_error(e.what());
    return FHEG_ERR_INTERNAL;
  }
}

FHEG_API void fheg_server_destroy(fheg_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (Slot& sl : s->slots) {
    cudaStreamDestroy(sl.stream);
    cudaEventDestroy(sl.done);
  }
  delete s;
}

FHEG_API int fheg_server_submit(fheg_server* s, const fheg_request* req, uint64_t* id) {
  try {
    fheg::set_last_error("");
    if (!s || !req || !id) throw Error(FHEG_ERR_INVALID_ARGUMENT, "null input");
    Req q;
    q.r = *req;
    describe(q);
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) throw Error(FHEG_ERR_INVALID_ARGUMENT, "server is stopping");
    q.id = s->next_id++;
    q.t_submit = now_ns();
    s->reqs.emplace(q.id, q);
    s->pending.push_back(q.id);
    s->submitted++;
    *id = q.id;
    s->cv_work.notify_one();
    return FHEG_OK;
  } catch (const Error& e) {
    fheg::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    fheg::set_last_error(e.what());
    return FHEG_ERR_INTERNAL;
  }
}

FHEG_API int fheg_server_wait(fheg_server* s, uint64_t id, uint32_t timeout_ms) {
  if (!s) return FHEG_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) {
    fheg::set_last_error("unknown request");
    return FHEG_ERR_INVALID_ARGUMENT;
  }
  const bool done = s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                                        [&] { return s->reqs.at(id).status >= 0; });
  if (!done) {
    fheg::set_last_error("request not finished within the timeout");
    return FHEG_ERR_TIMEOUT;
  }
  const Req& q = s->reqs.at(id);
  fheg::set_last_error(q.err);
  return q.status;
}

FHEG_API int fheg_server_request_times(fheg_server* s, uint64_t id, int64_t* submit_ns, int64_t* start_ns,
                                       int64_t* done_ns) {
  if (!s || !submit_ns || !start_ns || !done_ns) return FHEG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return FHEG_ERR_INVALID_ARGUMENT;
  *submit_ns = it->second.t_submit;
  *start_ns = it->second.t_start;
  *done_ns = it->second.t_done;
  return FHEG_OK;
}

FHEG_API int fheg_server_release(fheg_server* s, uint64_t id) {
  if (!s) return FHEG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end() || it->second.status < 0) return FHEG_ERR_INVALID_ARGUMENT;
  s->reqs.erase(it);
  return FHEG_OK;
}

FHEG_API int fheg_server_stats(fheg_server* s, uint64_t* submitted, uint64_t* completed, uint64_t* batches,
                               size_t* peak_bytes) {
  if (!s || !submitted || !completed || !batches || !peak_bytes) return FHEG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  *submitted = s->submitted;
  *completed = s->completed;
  *batches = s->batches;
  *peak_bytes = s->arena.peak;
  return FHEG_OK;
}
