// C ABI of libfheg (declarations and reference mapping in include/fheg.h).

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "fheg.h"
#include "abi_call.hpp"
#include "handles.hpp"
#include "lib.hpp"

using namespace fheg;

namespace {

thread_local std::string g_last_error;

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

BigUint big(const uint64_t* w, size_t n) { return w && n ? BigUint::from_words(w, n) : BigUint(); }

}  // namespace

namespace fheg {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace fheg

FHEG_API const char* fheg_version(void) { return "fheg 0.1.0 (sm_103a)"; }

FHEG_API const char* fheg_status_string(int s) {
  switch (s) {
    case FHEG_OK: return "ok";
    case FHEG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case FHEG_ERR_INVALID_MODULUS: return "invalid modulus";
    case FHEG_ERR_NTT_UNSUPPORTED: return "NTT not supported for this modulus and degree";
    case FHEG_ERR_INVALID_CONTEXT: return "invalid context";
    case FHEG_ERR_INVALID_LEVEL: return "invalid level";
    case FHEG_ERR_KEY_MISMATCH: return "key does not match the ciphertext";
    case FHEG_ERR_WRONG_PARTS: return "wrong number of ciphertext parts";
    case FHEG_ERR_NO_MORE_CONTEXT: return "no more context";
    case FHEG_ERR_BUDGET: return "memory budget exhausted";
    case FHEG_ERR_CUDA: return "CUDA error";
    case FHEG_ERR_TIMEOUT: return "timeout";
    case FHEG_ERR_UNSUPPORTED: return "unsupported";
    default: return "internal error";
  }
}

FHEG_API const char* fheg_last_error(void) { return g_last_error.c_str(); }

FHEG_API uint64_t fheg_kernel_launch_count(void) { return g_launches.load(); }

// ---------------------------------------------------------------------------
// Host-only number theory.

FHEG_API int fheg_generate_prime(uint32_t num_bits, uint64_t modulo, uint64_t upper_bound, uint64_t* out) {
  return abi_call([&] {
    abi_need(out != nullptr && modulo != 0, "null output or zero modulo");
    *out = generate_prime(num_bits, modulo, upper_bound);
  });
}

FHEG_API int fheg_supports_ntt(uint64_t p, size_t n) {
  if (n < 8 || (n & (n - 1))) return 0;
  return supports_ntt(p, n) ? 1 : 0;
}

FHEG_API int fheg_ntt_default_root(uint64_t p, size_t n, uint64_t* out_root) {
  return abi_call([&] {
    abi_need(out_root != nullptr, "null output");
    *out_root = default_ntt_root(p, n);
  });
}

FHEG_API int fheg_ntt_tables_host(uint64_t p, size_t n, uint64_t root, uint64_t* omegas, uint64_t* omegas_shoup,
                                  uint64_t* zetas_inv, uint64_t* zetas_inv_shoup, uint64_t* out_size_inv) {
  return abi_call([&] {
    abi_need(omegas && omegas_shoup && zetas_inv && zetas_inv_shoup && out_size_inv, "null output");
    NttTablesHost t = make_ntt_tables(p, n, root);
    std::memcpy(omegas, t.omegas.data(), n * 8);
    std::memcpy(omegas_shoup, t.omegas_shoup.data(), n * 8);
    std::memcpy(zetas_inv, t.zetas_inv.data(), n * 8);
    std::memcpy(zetas_inv_shoup, t.zetas_inv_shoup.data(), n * 8);
    out_size_inv[0] = t.size_inv;
    out_size_inv[1] = t.size_inv_shoup;
  });
}

FHEG_API int fheg_rns_scaler_constants_host(const uint64_t* from_moduli, size_t from_len, const uint64_t* to_moduli,
                                            size_t to_len, const uint64_t* num, size_t num_words,
                                            const uint64_t* den, size_t den_words, uint64_t* out,
                                            size_t out_words) {
  return abi_call([&] {
    abi_need(from_moduli && to_moduli && out && from_len && to_len, "null or empty input");
    const size_t F = from_len, T = to_len;
    abi_need(out_words >= 5 + 2 * T + 2 * T * F + 5 * F, "output too small");
    RnsContextHost from(std::vector<uint64_t>(from_moduli, from_moduli + F));
    RnsContextHost to(std::vector<uint64_t>(to_moduli, to_moduli + T));
    RnsScalerHost s = make_rns_scaler(from, to, big(num, num_words), big(den, den_words));
    size_t o = 0;
    out[o++] = s.theta_garner_shift;
    out[o++] = s.is_one ? 1 : 0;
    out[o++] = s.theta_gamma_lo;
    out[o++] = s.theta_gamma_hi;
    out[o++] = s.theta_gamma_sign ? 1 : 0;
    for (auto v : s.gamma) out[o++] = v;
    for (auto v : s.gamma_shoup) out[o++] = v;
    for (auto v : s.omega) out[o++] = v;
    for (auto v : s.omega_shoup) out[o++] = v;
    for (auto v : s.theta_omega_lo) out[o++] = v;
    for (auto v : s.theta_omega_hi) out[o++] = v;
    for (auto v : s.theta_omega_sign) out[o++] = v;
    for (auto v : s.theta_garner_lo) out[o++] = v;
    for (auto v : s.theta_garner_hi) out[o++] = v;
  });
}

// ---------------------------------------------------------------------------
// Contexts and polynomial operations.

FHEG_API int fheg_context_create(const uint64_t* moduli, size_t num_moduli, size_t degree, const uint64_t* roots,
                                 fheg_context** out) {
  return abi_call([&] {
    abi_need(moduli && num_moduli && out, "null or empty input");
    auto h = new fheg_context();
    try {
      h->c = std::make_shared<Context>(std::vector<uint64_t>(moduli, moduli + num_moduli), degree, roots);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_context_destroy(fheg_context* ctx) { delete ctx; }
FHEG_API size_t fheg_context_num_moduli(const fheg_context* ctx) { return ctx ? ctx->c->L() : 0; }
FHEG_API size_t fheg_context_degree(const fheg_context* ctx) { return ctx ? ctx->c->N() : 0; }

FHEG_API int fheg_ntt_forward(const fheg_context* ctx, uint64_t* d_polys, size_t count, int lazy, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && (d_polys || !count), "null input");
    PolyRef r = plain_ref(d_polys, ctx->c->L(), ctx->c->logn);
    ntt_forward(*ctx->c, r, r, count, lazy != 0, as_stream(stream));
  });
}

FHEG_API int fheg_ntt_backward(const fheg_context* ctx, uint64_t* d_polys, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && (d_polys || !count), "null input");
    PolyRef r = plain_ref(d_polys, ctx->c->L(), ctx->c->logn);
    ntt_backward(*ctx->c, r, r, count, as_stream(stream));
  });
}

FHEG_API int fheg_ntt_plan_set(uint32_t logn, uint32_t block_logn) {
  return abi_call([&] { set_ntt_block_logn(logn, block_logn); });
}

FHEG_API int fheg_ntt_prefetch_set(int on) {
  return abi_call([&] { set_ntt_prefetch(on != 0); });
}

FHEG_API int fheg_ntt_cluster_set(uint32_t logn, int on) {
  return abi_call([&] { set_ntt_cluster(logn, on != 0); });
}

FHEG_API int fheg_ntt_cluster_get(uint32_t logn, int* on) {
  return abi_call([&] {
    abi_need(on && logn <= 16, "bad size or null output");
    *on = ntt_cluster_enabled(logn) ? 1 : 0;
  });
}

FHEG_API int fheg_rns_tensor_set(int on) {
  return abi_call([&] { set_rns_tc(on != 0); });
}

FHEG_API int fheg_rns_tensor_get(int* on) {
  return abi_call([&] {
    abi_need(on, "null output");
    *on = rns_tc_enabled() ? 1 : 0;
  });
}

FHEG_API int fheg_rns_tensor_wait_failures(uint64_t* count) {
  return abi_call([&] {
    abi_need(count, "null output");
    *count = rns_tc_wait_failures();
  });
}

FHEG_API int fheg_ntt_plan_get(uint32_t logn, uint32_t* block_logn) {
  return abi_call([&] {
    abi_need(block_logn && logn >= 3 && logn <= 16, "bad size or null output");
    *block_logn = ntt_block_logn(logn);
  });
}

// Times `run` under every valid NTT plan for 2^logn (one warm-up pass, then
// a timed pass) and installs the fastest.
template <class F>
uint32_t autotune_plans(uint32_t logn, cudaStream_t st, F run) {
  // (block size, cluster mode) candidates.
  std::vector<std::pair<uint32_t, bool>> plans;
  for (uint32_t bl = 12; bl <= 14; bl++)
    if (bl <= logn && logn - bl <= 4 && (bl < logn || logn <= 14)) {
      plans.push_back({bl, false});
      if (bl == 12 && bl < logn) plans.push_back({bl, true});
    }
  const uint32_t before = ntt_block_logn(logn);
  const bool before_cluster = ntt_cluster_enabled(logn);
  if (plans.empty()) return before;
  cudaEvent_t e0, e1;
  check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
  check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
  float best_ms = 0;
  std::pair<uint32_t, bool> best{before, before_cluster};
  try {
    for (const auto& plan : plans) {
      set_ntt_block_logn(logn, plan.first);
      set_ntt_cluster(logn, plan.second);
      for (int rep = 0; rep < 2; rep++) {
        check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");
        run();
        check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
      }
      check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0;
      check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
      if (best_ms == 0 || ms < best_ms) {
        best_ms = ms;
        best = plan;
      }
    }
  } catch (...) {
    set_ntt_block_logn(logn, before);
    set_ntt_cluster(logn, before_cluster);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  set_ntt_block_logn(logn, best.first);
  set_ntt_cluster(logn, best.second);
  return best.first;
}

FHEG_API int fheg_ntt_autotune(const fheg_context* ctx, size_t count, void* stream, uint32_t* block_logn) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && count && block_logn, "null input");
    const Context& c = *ctx->c;
    cudaStream_t st = as_stream(stream);
    DevBuf buf(count * c.L() * c.N() * 8);
    check_cuda(cudaMemsetAsync(buf.ptr, 0, buf.bytes, st), "cudaMemsetAsync");
    PolyRef r = plain_ref(buf.u64(), c.L(), c.logn);
    *block_logn = autotune_plans(c.logn, st, [&] {
      for (int k = 0; k < 3; k++) {
        ntt_forward(c, r, r, count, false, st);
        ntt_backward(c, r, r, count, st);
      }
    });
  });
}

namespace {

// Event time of `run` on `st`: the fastest of three calls after a warm-up
// call (one call alone flips close choices on run-to-run noise).
template <class F>
float time_once(cudaStream_t st, F run) {
  cudaEvent_t e0, e1;
  check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
  check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
  float ms = 0;
  try {
    run();
    for (int k = 0; k < 3; k++) {
      check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");
      run();
      check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
      check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float t = 0;
      check_cuda(cudaEventElapsedTime(&t, e0, e1), "cudaEventElapsedTime");
      if (k == 0 || t < ms) ms = t;
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

void get_mul_plan(const Multiplicator& m, uint32_t* plan) {
  const uint32_t logn = m.base->logn, dflt = ntt_block_logn(logn);
  plan[0] = m.plan_a ? m.plan_a : dflt;
  plan[1] = m.plan_c ? m.plan_c : dflt;
  plan[2] = m.plan_d ? m.plan_d : dflt;
  plan[3] = m.plan_f ? m.plan_f : dflt;
  plan[4] = m.f_split ? 1 : 0;
  plan[5] = m.tensor_split ? 1 : 0;
}

void set_mul_plan(Multiplicator& m, const uint32_t* plan) {
  const uint32_t logn = m.base->logn;
  for (int k = 0; k < 4; k++)
    if (!ntt_plan_valid(logn, plan[k])) throw Error(FHEG_ERR_INVALID_ARGUMENT, "unsupported NTT plan");
  m.plan_a = plan[0];
  m.plan_c = plan[1];
  m.plan_d = plan[2];
  m.plan_f = plan[3];
  m.f_split = plan[4] != 0;
  m.tensor_split = plan[5] != 0;
}

}  // namespace

FHEG_API int fheg_multiplicator_stage_times(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                            uint64_t* d_out, size_t count, void* stream, float* ms) {
  return abi_call([&] {
    abi_count(count);
    abi_need(m && d_lhs && d_rhs && d_out && count && ms, "null input");
    cudaStream_t st = as_stream(stream);
    cudaEvent_t ev[8] = {};
    try {
      for (auto& e : ev) check_cuda(cudaEventCreate(&e), "cudaEventCreate");
      m->m->multiply(d_lhs, d_rhs, d_out, count, st, nullptr, ev);
      check_cuda(cudaEventSynchronize(ev[7]), "cudaEventSynchronize");
      for (int k = 0; k < 7; k++) check_cuda(cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]), "cudaEventElapsedTime");
    } catch (...) {
      for (auto& e : ev)
        if (e) cudaEventDestroy(e);
      throw;
    }
    for (auto& e : ev) cudaEventDestroy(e);
  });
}

FHEG_API int fheg_multiplicator_set_small_plan(fheg_multiplicator* m, size_t max_count, const uint32_t* plan) {
  return abi_call([&] {
    abi_need(m && (plan || !max_count), "null input");
    Multiplicator& mm = *m->m;
    if (max_count) {
      for (int k = 0; k < 4; k++)
        if (!ntt_plan_valid(mm.base->logn, plan[k])) throw Error(FHEG_ERR_INVALID_ARGUMENT, "unsupported NTT plan");
      std::copy(plan, plan + 6, mm.small_plan);
    }
    mm.small_count = max_count;
  });
}

FHEG_API int fheg_multiplicator_get_plan(const fheg_multiplicator* m, uint32_t* plan) {
  return abi_call([&] {
    abi_need(m && plan, "null input");
    get_mul_plan(*m->m, plan);
  });
}

FHEG_API int fheg_multiplicator_set_plan(fheg_multiplicator* m, const uint32_t* plan) {
  return abi_call([&] {
    abi_need(m && plan, "null input");
    set_mul_plan(*m->m, plan);
  });
}

FHEG_API int fheg_multiplicator_autotune(fheg_multiplicator* m, size_t count, void* stream, uint32_t* plan) {
  return abi_call([&] {
    abi_count(count);
    abi_need(m && count, "null input");
    Multiplicator& mult = *m->m;
    const Context& bc = *mult.base;
    cudaStream_t st = as_stream(stream);
    const size_t in_words = count * 2 * bc.L() * bc.N();
    const size_t out_words = count * mult.out_parts() * mult.par->ctx(mult.out_level())->L() * bc.N();
    DevBuf buf((2 * in_words + out_words) * 8);
    check_cuda(cudaMemsetAsync(buf.ptr, 0, buf.bytes, st), "cudaMemsetAsync");
    uint64_t* lhs = buf.u64();
    auto run = [&] { mult.multiply(lhs, lhs + in_words, lhs + 2 * in_words, count, st); };
    // Batches the small-batch plan covers tune that plan; others the main one.
    bool small = count <= mult.small_count;
    for (int k = 0; k < 4; k++) small = small && ntt_plan_valid(bc.logn, mult.small_plan[k]);
    auto get = [&](uint32_t* p) {
      if (small) std::copy(mult.small_plan, mult.small_plan + 6, p);
      else get_mul_plan(mult, p);
    };
    auto set = [&](const uint32_t* p) {
      if (small) std::copy(p, p + 6, mult.small_plan);
      else set_mul_plan(mult, p);
    };
    // Coordinate descent over the stages, starting from the current plan.
    uint32_t cur[6];
    get(cur);
    set(cur);
    float best = time_once(st, run);
    const std::vector<uint32_t> plans = ntt_plans(bc.logn);
    auto consider = [&](const uint32_t* cand) {
      if (std::equal(cand, cand + 6, cur)) return;
      set(cand);
      const float ms = time_once(st, run);
      if (ms < best) {
        best = ms;
        std::copy(cand, cand + 6, cur);
      }
    };
    for (int k = 0; k < 4; k++) {
      for (uint32_t bl : plans) {
        for (uint32_t split = 0; split < 2u; split++) {
          if (split && !(k == 3 && bl >= bc.logn) && k != 2) continue;
          uint32_t cand[6];
          std::copy(cur, cur + 6, cand);
          cand[k] = bl;
          if (k == 3) cand[4] = split;
          if (k == 2) cand[5] = split;
          consider(cand);
        }
      }
    }
    set(cur);
    if (plan) std::copy(cur, cur + 6, plan);
  });
}

FHEG_API int fheg_poly_scalar_mul(const fheg_context* ctx, const uint64_t* scalar, size_t scalar_words,
                                  const uint64_t* d_in, uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_in && d_out) || !count), "null input");
    const Context& c = *ctx->c;
    poly_scalar_mul(c, big(scalar, scalar_words), plain_ref(const_cast<uint64_t*>(d_in), c.L(), c.logn),
                    plain_ref(d_out, c.L(), c.logn), count, as_stream(stream));
  });
}

FHEG_API int fheg_device_alloc(size_t bytes, void** out) {
  return abi_call([&] {
    abi_need(out != nullptr, "null output");
    *out = nullptr;
    if (bytes) check_cuda(cudaMalloc(out, bytes), "cudaMalloc");
  });
}

FHEG_API int fheg_device_free(void* ptr) {
  return abi_call([&] {
    if (ptr) check_cuda(cudaFree(ptr), "cudaFree");
  });
}

FHEG_API int fheg_copy_to_device(void* d_dst, const void* h_src, size_t bytes, void* stream) {
  return abi_call([&] {
    abi_need((d_dst && h_src) || !bytes, "null input");
    if (!bytes) return;
    check_cuda(cudaMemcpyAsync(d_dst, h_src, bytes, cudaMemcpyHostToDevice, as_stream(stream)), "H2D");
  });
}

FHEG_API int fheg_copy_to_host(void* h_dst, const void* d_src, size_t bytes, void* stream) {
  return abi_call([&] {
    abi_need((h_dst && d_src) || !bytes, "null input");
    if (!bytes) return;
    cudaStream_t st = as_stream(stream);
    check_cuda(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, st), "D2H");
    check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  });
}

FHEG_API int fheg_poly_op(const fheg_context* ctx, int op, const uint64_t* d_a, const uint64_t* d_b, uint64_t* d_out,
                          size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && op >= 0 && op <= 3, "bad context or op");
    abi_need((d_a && d_out && (op == 3 || d_b)) || !count, "null input");
    const Context& c = *ctx->c;
    PolyRef a = plain_ref(const_cast<uint64_t*>(d_a), c.L(), c.logn);
    PolyRef b = plain_ref(const_cast<uint64_t*>(d_b ? d_b : d_a), c.L(), c.logn);
    PolyRef o = plain_ref(d_out, c.L(), c.logn);
    poly_op(c, op, a, b, o, count, as_stream(stream));
  });
}

FHEG_API int fheg_poly_compute_shoup(const fheg_context* ctx, const uint64_t* d_polys, uint64_t* d_shoup,
                                     size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_polys && d_shoup) || !count), "null input");
    const Context& c = *ctx->c;
    poly_compute_shoup(c, plain_ref(const_cast<uint64_t*>(d_polys), c.L(), c.logn), plain_ref(d_shoup, c.L(), c.logn),
                       count, as_stream(stream));
  });
}

FHEG_API int fheg_poly_mul_shoup(const fheg_context* ctx, const uint64_t* d_a, const uint64_t* d_b,
                                 const uint64_t* d_b_shoup, uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_a && d_b && d_b_shoup && d_out) || !count), "null input");
    const Context& c = *ctx->c;
    poly_mul_shoup(c, plain_ref(const_cast<uint64_t*>(d_a), c.L(), c.logn),
                   plain_ref(const_cast<uint64_t*>(d_b), c.L(), c.logn),
                   plain_ref(const_cast<uint64_t*>(d_b_shoup), c.L(), c.logn), plain_ref(d_out, c.L(), c.logn), count,
                   as_stream(stream));
  });
}

FHEG_API int fheg_poly_substitute(const fheg_context* ctx, size_t exponent, int representation, const uint64_t* d_in,
                                  uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_in && d_out) || !count), "null input");
    abi_need(d_in != d_out || !count, "d_out must not alias d_in");
    const Context& c = *ctx->c;
    PolyRef i = plain_ref(const_cast<uint64_t*>(d_in), c.L(), c.logn);
    PolyRef o = plain_ref(d_out, c.L(), c.logn);
    poly_substitute(c, exponent, representation != 0, i, o, count, as_stream(stream));
  });
}

FHEG_API int fheg_poly_switch_down(const fheg_context* ctx, int representation, uint64_t* d_in, uint64_t* d_out,
                                   size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_in && d_out) || !count), "null input");
    const Context& c = *ctx->c;
    PolyRef i = plain_ref(d_in, c.L(), c.logn);
    PolyRef o = plain_ref(d_out, c.L() - 1, c.logn);
    if (representation) poly_switch_down_ntt(c, i, o, count, as_stream(stream));
    else poly_switch_down_pb(c, i, o, count, as_stream(stream));
  });
}

FHEG_API int fheg_scaler_create(const fheg_context* from, const fheg_context* to, const uint64_t* num,
                                size_t num_words, const uint64_t* den, size_t den_words, fheg_scaler** out) {
  return abi_call([&] {
    abi_need(from && to && out, "null input");
    BigUint d = big(den, den_words);
    abi_need(!d.is_zero(), "ScalingFactor denominator is zero");
    auto h = new fheg_scaler();
    try {
      h->s.reset(new Scaler(from->c, to->c, big(num, num_words), d));
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_scaler_destroy(fheg_scaler* s) { delete s; }

FHEG_API int fheg_scaler_scale(const fheg_scaler* s, int representation, const uint64_t* d_in, uint64_t* d_out,
                               size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(s && ((d_in && d_out) || !count), "null input");
    abi_need(d_in != d_out || !count, "d_out must not alias d_in");
    const Scaler& sc = *s->s;
    PolyRef i = plain_ref(const_cast<uint64_t*>(d_in), sc.from->L(), sc.from->logn);
    PolyRef o = plain_ref(d_out, sc.to->L(), sc.to->logn);
    fheg_scaler* ms = const_cast<fheg_scaler*>(s);
    if (representation) ms->scratch.reserve(count * sc.from->L() * sc.from->N() * 8);
    scaler_scale(sc, representation != 0, i, o, count, ms->scratch.u64(), as_stream(stream));
  });
}

// ---------------------------------------------------------------------------
// BFV

FHEG_API int fheg_params_create(size_t degree, const uint64_t* moduli, size_t num_moduli, uint64_t plaintext,
                                fheg_params** out) {
  return abi_call([&] {
    abi_need(moduli && num_moduli && out, "null or empty input");
    auto h = new fheg_params();
    try {
      h->p.reset(new Params(degree, std::vector<uint64_t>(moduli, moduli + num_moduli), plaintext));
      for (auto& c : h->p->levels) h->level_handles.push_back(fheg_context{c});
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_params_destroy(fheg_params* par) { delete par; }

FHEG_API int fheg_params_context_at_level(const fheg_params* par, size_t level, const fheg_context** out) {
  return abi_call([&] {
    abi_need(par && out, "null input");
    if (level > par->p->max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    *out = &par->level_handles[level];
  });
}

FHEG_API size_t fheg_params_max_level(const fheg_params* par) { return par ? par->p->max_level() : 0; }

// A key-switching key with room for c0 and c1, c0 uploaded from h_c0 unless
// it is null (shared by the plain, seeded and message constructors).
fheg_ksk* new_ksk_handle(const fheg_params* par, size_t ciphertext_level, size_t ksk_level, const uint64_t* h_c0,
                         size_t count, int64_t log_base) {
  const Params& p = *par->p;
  if (ciphertext_level > p.max_level() || ksk_level > p.max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
  if (ksk_level > ciphertext_level) throw Error(FHEG_ERR_INVALID_LEVEL, "Unexpected levels");
  auto h = new fheg_ksk();
  try {
    Ksk& k = h->k;
    k.par = &p;
    k.ciphertext_level = ciphertext_level;
    k.ksk_level = ksk_level;
    k.ctx_ct = p.ctx(ciphertext_level);
    k.ctx_ksk = p.ctx(ksk_level);
    if (log_base < 0) log_base = k.ctx_ksk->L() == 1 ? log_modulus_of(k.ctx_ksk->moduli[0]) / 2 : 0;
    if (log_base > 0) {
      // key_switching_key.rs:63-89, 360-372: the base-2^log_base digits of a
      // single-modulus ciphertext, against a key at the last level.
      if (ksk_level != p.max_level() || ciphertext_level != p.max_level())
        throw Error(FHEG_ERR_INVALID_LEVEL, "A decomposition size is specified but the levels are not maximal");
      if (log_base > 62) throw Error(FHEG_ERR_INVALID_ARGUMENT, "decomposition base above 2^62");
      const uint32_t lm = log_modulus_of(k.ctx_ksk->moduli[0]);
      if (count != (lm + log_base - 1) / log_base)
        throw Error(FHEG_ERR_KEY_MISMATCH, "count must equal the decomposition's digits");
      k.log_base = (uint32_t)log_base;
    } else if (count != k.ctx_ct->L()) {
      throw Error(FHEG_ERR_KEY_MISMATCH, "count must equal the ciphertext moduli");
    }
    k.count = count;
    ksk_build_switch_chain(k);
    const size_t words = count * k.ctx_ksk->L() * k.ctx_ksk->N();
    k.keys.alloc(2 * words * 8);
    if (h_c0) upload(k.values(0), h_c0, words * 8);
  } catch (...) {
    delete h;
    throw;
  }
  return h;
}

FHEG_API int fheg_ksk_create(const fheg_params* par, size_t ciphertext_level, size_t ksk_level, const uint64_t* h_c0,
                             const uint64_t* h_c1, size_t count, fheg_ksk** out) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && h_c0 && h_c1 && out, "null input");
    fheg_ksk* h = new_ksk_handle(par, ciphertext_level, ksk_level, h_c0, count);
    try {
      const Ksk& k = h->k;
      upload(k.values(1), h_c1, count * k.ctx_ksk->L() * k.ctx_ksk->N() * 8);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API int fheg_ksk_create_seeded(const fheg_params* par, size_t ciphertext_level, size_t ksk_level,
                                    const uint64_t* h_c0, const uint8_t* seed, size_t count, fheg_ksk** out) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && h_c0 && seed && out, "null input");
    fheg_ksk* h = new_ksk_handle(par, ciphertext_level, ksk_level, h_c0, count);
    try {
      Ksk& k = h->k;
      k.seed.assign(seed, seed + 32);
      const std::vector<uint8_t> seeds = ksk_c1_seeds(seed, count);
      DevBuf d_seeds(seeds.size());
      upload(d_seeds.ptr, seeds.data(), seeds.size());
      Workspace ws;
      poly_random_from_seed(*k.ctx_ksk, static_cast<const uint8_t*>(d_seeds.ptr), k.values(1),
                            k.ctx_ksk->L() * k.ctx_ksk->N(), count, ws, nullptr);
      check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_ksk_destroy(fheg_ksk* k) { delete k; }

FHEG_API int fheg_relinearize(const fheg_ksk* rk, const uint64_t* d_ct3, uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(rk && ((d_ct3 && d_out) || !count), "null input");
    relinearize(rk->k, d_ct3, d_out, count, rk->k.ws, as_stream(stream));
  });
}

FHEG_API int fheg_galois_relinearize(const fheg_ksk* gk, size_t exponent, const uint64_t* d_ct, uint64_t* d_out,
                                     size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(gk && ((d_ct && d_out) || !count), "null input");
    abi_need(d_ct != d_out || !count, "d_out must not alias d_ct");
    galois_relinearize(gk->k, exponent, d_ct, d_out, count, gk->k.ws, as_stream(stream));
  });
}

FHEG_API int fheg_rgsw_create(const fheg_params* par, size_t level, const uint64_t* h_ksk0_c0,
                              const uint64_t* h_ksk0_c1, const uint64_t* h_ksk1_c0, const uint64_t* h_ksk1_c1,
                              fheg_rgsw** out) {
  return abi_call([&] {
    abi_need(par && h_ksk0_c0 && h_ksk0_c1 && h_ksk1_c0 && h_ksk1_c1 && out, "null input");
    const Params& p = *par->p;
    if (level > p.max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    auto h = new fheg_rgsw();
    try {
      Ksk& k = h->k;
      k.par = &p;
      k.ciphertext_level = k.ksk_level = level;
      k.ctx_ct = k.ctx_ksk = p.ctx(level);
      const size_t L = k.ctx_ct->L();
      if (L < 2) throw Error(FHEG_ERR_UNSUPPORTED, "These parameters do not support key switching");
      k.count = 2 * L;
      // [part][digit][L][N]: digits 0..L-1 from ksk0, L..2L-1 from ksk1.
      const size_t words = L * L * k.ctx_ct->N();
      k.keys.alloc(4 * words * 8);
      upload(k.values(0), h_ksk0_c0, words * 8);
      upload(k.values(0) + words, h_ksk1_c0, words * 8);
      upload(k.values(1), h_ksk0_c1, words * 8);
      upload(k.values(1) + words, h_ksk1_c1, words * 8);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_rgsw_destroy(fheg_rgsw* rgsw) { delete rgsw; }

FHEG_API int fheg_external_product(const fheg_rgsw* rgsw, const uint64_t* d_ct, uint64_t* d_out, size_t count,
                                   void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(rgsw && ((d_ct && d_out) || !count), "null input");
    external_product(rgsw->k, d_ct, d_out, count, rgsw->k.ws, as_stream(stream));
  });
}

FHEG_API int fheg_galois_relinearize_batch(const fheg_params* par, const fheg_ksk* const* keys,
                                           const size_t* exponents, const uint64_t* const* d_cts,
                                           uint64_t* const* d_outs, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((keys && exponents && d_cts && d_outs) || !count), "null input");
    std::vector<RotRequest> req(count);
    for (size_t b = 0; b < count; b++) {
      abi_need(keys[b] && d_cts[b] && d_outs[b] && d_cts[b] != d_outs[b], "null or aliased batch entry");
      req[b] = RotRequest{&keys[b]->k, exponents[b], d_cts[b], d_outs[b]};
    }
    fheg_params* ph = const_cast<fheg_params*>(par);
    cudaStream_t st = as_stream(stream);
    // Every request is checked before the first launch, so an invalid one in
    // the second half cannot leave the first half's outputs written.
    validate_rot_requests(*par->p, req.data(), count);
    if (count < 16) {
      galois_relinearize_batch(*par->p, req.data(), count, ph->ws, st);
      return;
    }
    // Two halves side by side, the second on the parameters' own stream
    // between a fork and a join on the caller's stream (as the batched
    // multiplication does).
    if (!ph->side) check_cuda(cudaStreamCreateWithFlags(&ph->side, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!ph->fork) check_cuda(cudaEventCreateWithFlags(&ph->fork, cudaEventDisableTiming), "cudaEventCreate");
    if (!ph->join) check_cuda(cudaEventCreateWithFlags(&ph->join, cudaEventDisableTiming), "cudaEventCreate");
    const size_t c0 = count / 2;
    check_cuda(cudaEventRecord(ph->fork, st), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(ph->side, ph->fork, 0), "cudaStreamWaitEvent");
    galois_relinearize_batch(*par->p, req.data(), c0, ph->ws, st);
    galois_relinearize_batch(*par->p, req.data() + c0, count - c0, ph->side_ws, ph->side);
    check_cuda(cudaEventRecord(ph->join, ph->side), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(st, ph->join, 0), "cudaStreamWaitEvent");
  });
}

FHEG_API int fheg_ciphertext_switch_down(const fheg_params* par, size_t level, size_t parts, uint64_t* d_ct,
                                         uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && parts >= 1 && ((d_ct && d_out) || !count), "null input");
    ciphertext_switch_down(*par->p, level, parts, d_ct, d_out, count, as_stream(stream));
  });
}

FHEG_API int fheg_ciphertext_switch_to_level(const fheg_params* par, size_t level, size_t target_level,
                                             size_t parts, uint64_t* d_ct, uint64_t* d_out, size_t count,
                                             void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((d_ct && d_out) || !count), "null input");
    const Params& p = *par->p;
    if (target_level < level || target_level > p.max_level())
      throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    cudaStream_t st = as_stream(stream);
    const size_t N = p.degree;
    if (target_level == level) {
      const size_t bytes = count * parts * p.ctx(level)->L() * N * 8;
      if (bytes) check_cuda(cudaMemcpyAsync(d_out, d_ct, bytes, cudaMemcpyDeviceToDevice, st), "D2D");
      return;
    }
    // ciphertext.rs:100-119: one switch_down per level. Intermediate levels
    // alternate between a scratch region of the parameters' workspace and
    // d_ct (consumed as scratch, large enough for every lower level).
    Workspace& ws = const_cast<fheg_params*>(par)->ws;
    ws.reserve(count * parts * (p.ctx(level)->L() - 1) * N * 8);
    uint64_t* src = d_ct;
    for (size_t l = level; l < target_level; l++) {
      uint64_t* dst = (l + 1 == target_level) ? d_out : (src == d_ct ? ws.base() : d_ct);
      ciphertext_switch_down(p, l, parts, src, dst, count, st);
      src = dst;
    }
  });
}

FHEG_API int fheg_ciphertext_add(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_a,
                                 const uint64_t* d_b, uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((d_a && d_b && d_out) || !count), "null input");
    const Context& c = *par->p->ctx(level);
    PolyRef a = plain_ref(const_cast<uint64_t*>(d_a), c.L(), c.logn);
    PolyRef b = plain_ref(const_cast<uint64_t*>(d_b), c.L(), c.logn);
    PolyRef o = plain_ref(d_out, c.L(), c.logn);
    poly_op(c, 0, a, b, o, count * parts, as_stream(stream));
  });
}

FHEG_API int fheg_multiplicator_create_default(const fheg_ksk* rk, fheg_multiplicator** out) {
  return abi_call([&] {
    abi_need(rk && out, "null input");
    auto h = new fheg_multiplicator();
    try {
      h->m = make_default_multiplicator(rk->k);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API int fheg_multiplicator_create(const fheg_params* par, size_t level, const uint64_t* lhs_num,
                                       size_t lhs_num_words, const uint64_t* lhs_den, size_t lhs_den_words,
                                       const uint64_t* rhs_num, size_t rhs_num_words, const uint64_t* rhs_den,
                                       size_t rhs_den_words, const uint64_t* extended_basis, size_t extended_len,
                                       const uint64_t* post_num, size_t post_num_words, const uint64_t* post_den,
                                       size_t post_den_words, fheg_multiplicator** out) {
  return abi_call([&] {
    abi_need(par && extended_basis && extended_len && out, "null input");
    BigUint ld = big(lhs_den, lhs_den_words), rd = big(rhs_den, rhs_den_words), pd = big(post_den, post_den_words);
    abi_need(!ld.is_zero() && !rd.is_zero() && !pd.is_zero(), "ScalingFactor denominator is zero");
    auto h = new fheg_multiplicator();
    try {
      h->m = make_multiplicator(*par->p, level, big(lhs_num, lhs_num_words), ld, big(rhs_num, rhs_num_words), rd,
                                std::vector<uint64_t>(extended_basis, extended_basis + extended_len),
                                big(post_num, post_num_words), pd);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

FHEG_API void fheg_multiplicator_destroy(fheg_multiplicator* m) { delete m; }

FHEG_API int fheg_multiplicator_enable_relinearization(fheg_multiplicator* m, const fheg_ksk* rk) {
  return abi_call([&] {
    abi_need(m && rk, "null input");
    // mul.rs:133-142
    if (!rk->k.ctx_ct->same_as(*m->m->base) || rk->k.par != m->m->par)
      throw Error(FHEG_ERR_KEY_MISMATCH, "Invalid relinearization key context");
    m->m->rk = &rk->k;
  });
}

FHEG_API int fheg_multiplicator_enable_mod_switching(fheg_multiplicator* m) {
  return abi_call([&] {
    abi_need(m != nullptr, "null input");
    // mul.rs:146-155
    if (m->m->level >= m->m->par->max_level())
      throw Error(FHEG_ERR_NO_MORE_CONTEXT, "Cannot modulo switch as this is already the last level");
    m->m->mod_switch = true;
  });
}

FHEG_API int fheg_multiplicator_output_shape(const fheg_multiplicator* m, size_t* parts, size_t* level) {
  return abi_call([&] {
    abi_need(m && parts && level, "null input");
    *parts = m->m->out_parts();
    *level = m->m->out_level();
  });
}

FHEG_API int fheg_multiplicator_multiply(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                         uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(m && ((d_lhs && d_rhs && d_out) || !count), "null input");
    cudaStream_t st = as_stream(stream);
    Multiplicator& mm = *m->m;
    if (count < 32) {
      mm.multiply(d_lhs, d_rhs, d_out, count, st);
      return;
    }
    // Two halves side by side, the second on the multiplicator's own stream
    // between a fork and a join on the caller's stream (so the call stays
    // ordered on `stream`, and can be recorded into a graph): the branches
    // fill one another's barriers, tails and latency-bound phases.
    if (!m->side) check_cuda(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!m->fork) check_cuda(cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming), "cudaEventCreate");
    if (!m->join) check_cuda(cudaEventCreateWithFlags(&m->join, cudaEventDisableTiming), "cudaEventCreate");
    const size_t N = mm.base->N(), L = mm.base->L();
    const size_t in_pair = 2 * L * N, out_pair = mm.out_parts() * (mm.mod_switch ? L - 1 : L) * N;
    const size_t c0 = count / 2;
    check_cuda(cudaEventRecord(m->fork, st), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(m->side, m->fork, 0), "cudaStreamWaitEvent");
    mm.multiply(d_lhs, d_rhs, d_out, c0, st);
    mm.multiply(d_lhs + c0 * in_pair, d_rhs + c0 * in_pair, d_out + c0 * out_pair, count - c0, m->side, &m->side_ws);
    check_cuda(cudaEventRecord(m->join, m->side), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(st, m->join, 0), "cudaStreamWaitEvent");
  });
}

FHEG_API int fheg_multiply_groups(fheg_multiplicator* const* mults, const uint64_t* const* d_lhs,
                                  const uint64_t* const* d_rhs, uint64_t* const* d_out, const size_t* counts,
                                  size_t groups, void* stream) {
  return abi_call([&] {
    abi_need((mults && d_lhs && d_rhs && d_out && counts) || !groups, "null input");
    for (size_t g = 0; g < groups; g++) {
      abi_need(mults[g] && ((d_lhs[g] && d_rhs[g] && d_out[g]) || !counts[g]), "null group entry");
      for (size_t h = 0; h < g; h++)
        abi_need(mults[h] != mults[g], "a multiplicator appears in two groups (merge them into one batch)");
    }
    cudaStream_t st = as_stream(stream);
    // Every group on its multiplicator's own stream, forked from and joined
    // back into `st`: the groups' kernels overlap on the GPU and the call
    // stays ordered on `st`.
    cudaEvent_t fork = nullptr;
    check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
    struct EventGuard {
      cudaEvent_t e;
      ~EventGuard() { cudaEventDestroy(e); }
    } guard{fork};
    check_cuda(cudaEventRecord(fork, st), "cudaEventRecord");
    for (size_t g = 0; g < groups; g++) {
      fheg_multiplicator* m = mults[g];
      if (!m->side) check_cuda(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking), "cudaStreamCreate");
      if (!m->join) check_cuda(cudaEventCreateWithFlags(&m->join, cudaEventDisableTiming), "cudaEventCreate");
      check_cuda(cudaStreamWaitEvent(m->side, fork, 0), "cudaStreamWaitEvent");
      m->m->multiply(d_lhs[g], d_rhs[g], d_out[g], counts[g], m->side);
      check_cuda(cudaEventRecord(m->join, m->side), "cudaEventRecord");
    }
    for (size_t g = 0; g < groups; g++) check_cuda(cudaStreamWaitEvent(st, mults[g]->join, 0), "cudaStreamWaitEvent");
  });
}

FHEG_API int fheg_multiplicator_set_host_pipeline(fheg_multiplicator* m, size_t chunk, int streams) {
  return abi_call([&] {
    abi_need(m && streams >= 1 && streams <= fheg_multiplicator::kPipe, "null multiplicator or streams outside 1..4");
    m->host_chunk = chunk;
    m->host_streams = streams;
  });
}

FHEG_API int fheg_multiplicator_multiply_host(fheg_multiplicator* m, const uint64_t* h_lhs, const uint64_t* h_rhs,
                                              uint64_t* h_out, size_t count) {
  return abi_call([&] {
    abi_count(count);
    abi_need(m && ((h_lhs && h_rhs && h_out) || !count), "null input");
    if (!count) return;
    Multiplicator& mm = *m->m;
    const size_t N = mm.base->N(), L = mm.base->L();
    const size_t in_words = count * 2 * L * N;
    const size_t out_L = mm.mod_switch ? L - 1 : L;
    const size_t out_words = count * mm.out_parts() * out_L * N;
    mm.staging.reserve((2 * in_words + out_words) * 8);
    uint64_t* d_lhs = mm.staging.u64();
    uint64_t* d_rhs = d_lhs + in_words;
    uint64_t* d_out = d_rhs + in_words;
    const int ns = m->host_streams;
    for (int k = 0; k < ns; k++)
      if (!m->pipe[k]) check_cuda(cudaStreamCreateWithFlags(&m->pipe[k], cudaStreamNonBlocking), "stream");
    if (!m->copy_in) check_cuda(cudaStreamCreateWithFlags(&m->copy_in, cudaStreamNonBlocking), "stream");
    if (!m->copy_out) check_cuda(cudaStreamCreateWithFlags(&m->copy_out, cudaStreamNonBlocking), "stream");
    // Every chunk's inputs cross the host link back to back on one stream and
    // its output on another, in chunk order; chunk i multiplies on compute
    // stream i % ns once its inputs have landed. Each chunk has its own
    // staging rows, so no copy waits for a multiplication other than its
    // own chunk's, and no multiplication for a copy of another chunk. Small
    // chunks (4 pairs, three at a time) keep the fill (one chunk's inputs)
    // and the drain (one chunk's output) short.
    const size_t chunk = m->host_chunk ? std::min(m->host_chunk, count) : (count >= 8 ? 4 : count);
    const size_t nchunks = (count + chunk - 1) / chunk;
    for (cudaEvent_t* e : {&m->copied, &m->computed})
      if (!*e) check_cuda(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
    const size_t in_pair = 2 * L * N, out_pair = mm.out_parts() * out_L * N;
    // A chunk that fails to launch ends the call only once the copies already
    // queued have finished: none of them may write into h_out after the
    // caller regains it.
    auto drain = [&] {
      cudaStreamSynchronize(m->copy_in);
      for (int k = 0; k < ns; k++) cudaStreamSynchronize(m->pipe[k]);
      cudaStreamSynchronize(m->copy_out);
    };
    try {
      for (size_t i = 0; i < nchunks; i++) {
        const size_t first = i * chunk, c = std::min(chunk, count - first);
        const int k = (int)(i % ns);
        cudaStream_t st = m->pipe[k];
        check_cuda(cudaMemcpyAsync(d_lhs + first * in_pair, h_lhs + first * in_pair, c * in_pair * 8,
                                   cudaMemcpyHostToDevice, m->copy_in), "H2D");
        check_cuda(cudaMemcpyAsync(d_rhs + first * in_pair, h_rhs + first * in_pair, c * in_pair * 8,
                                   cudaMemcpyHostToDevice, m->copy_in), "H2D");
        check_cuda(cudaEventRecord(m->copied, m->copy_in), "cudaEventRecord");
        check_cuda(cudaStreamWaitEvent(st, m->copied, 0), "cudaStreamWaitEvent");
        mm.multiply(d_lhs + first * in_pair, d_rhs + first * in_pair, d_out + first * out_pair, c, st,
                    &m->pipe_ws[k]);
        check_cuda(cudaEventRecord(m->computed, st), "cudaEventRecord");
        check_cuda(cudaStreamWaitEvent(m->copy_out, m->computed, 0), "cudaStreamWaitEvent");
        check_cuda(cudaMemcpyAsync(h_out + first * out_pair, d_out + first * out_pair, c * out_pair * 8,
                                   cudaMemcpyDeviceToHost, m->copy_out), "D2H");
      }
    } catch (...) {
      drain();
      throw;
    }
    // The output stream waits for every chunk, and every chunk for its inputs.
    check_cuda(cudaStreamSynchronize(m->copy_out), "cudaStreamSynchronize");
    for (int k = 0; k < ns; k++) check_cuda(cudaStreamSynchronize(m->pipe[k]), "cudaStreamSynchronize");
    check_cuda(cudaStreamSynchronize(m->copy_in), "cudaStreamSynchronize");
  });
}
