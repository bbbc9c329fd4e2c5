// Internal object model of libfheg (the C ABI in include/fheg.h wraps these).
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "host_math.hpp"

namespace fheg {

// Owning device buffer.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  DevBuf() {}
  explicit DevBuf(size_t b) { alloc(b); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void alloc(size_t b) {
    release();
    if (b) check_cuda(cudaMalloc(&ptr, b), "cudaMalloc");
    bytes = b;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  // Grows (never shrinks) to at least b bytes; contents are not preserved.
  void reserve(size_t b) {
    if (b > bytes) alloc(b);
  }
  uint64_t* u64() const { return static_cast<uint64_t*>(ptr); }
};

void upload(void* dst, const void* src, size_t bytes);
// Sets the message returned by fheg_last_error() on this thread.
void set_last_error(const std::string& msg);

// NTT tables of one prime for one degree, resident on one device. Shared by
// every context that uses the prime (registry keyed by device, p, n, root).
struct PrimeTables {
  NttTablesHost host;
  DevBuf tables;  // 4 * n words: (omega, shoup) pairs, then (zeta_inv, shoup) pairs
  DevPrime dev;
};
std::shared_ptr<PrimeTables> get_prime_tables(uint64_t p, size_t n, uint64_t root);

// rq::Context (fhe-math/src/rq/context.rs:9-19) on the device.
struct Context {
  size_t degree = 0;
  uint32_t logn = 0;
  std::vector<uint64_t> moduli;
  std::vector<std::shared_ptr<PrimeTables>> primes;
  DevBuf d_primes;  // DevPrime[L]
  // rq/context.rs:66-73: inv_last_qi_mod_qj and Shoup values for i < L-1,
  // followed by (q_i - (floor(q_last/2) mod q_i)) for i < L-1.
  DevBuf d_switch;
  std::unique_ptr<RnsContextHost> rns;
  int device = 0;

  Context(const std::vector<uint64_t>& moduli, size_t degree, const uint64_t* roots);
  size_t L() const { return moduli.size(); }
  size_t N() const { return degree; }
  const DevPrime* primes_dev() const { return static_cast<const DevPrime*>(d_primes.ptr); }
  std::vector<uint64_t> roots() const;
  bool same_as(const Context& o) const { return degree == o.degree && moduli == o.moduli; }
  // Context with the first `count` moduli (the same roots).
  std::shared_ptr<Context> prefix(size_t count) const;
};

// rns::RnsScaler (fhe-math/src/rns/scaler.rs:51-72): the host constants and
// the per-target-modulus values each launch copies into its parameters.
struct RnsScalerD {
  RnsScalerHost host;
  std::vector<uint64_t> gamma_neg;     // (q_j - gamma_j) mod q_j
  std::vector<uint64_t> gamma_neg_hi;  // gamma_neg * 2^62 mod q_j
  std::vector<uint64_t> to_moduli, to_bhi, to_blo;
  // Montgomery forms (times 2^64 mod q_j) of omega (row j: to_len x from_len),
  // gamma_neg and gamma_neg_hi, and -q_j^-1 mod 2^64; set when every target
  // modulus is odd (mont).
  bool mont = false;
  std::vector<uint64_t> omega_mont, gamma_neg_mont, gamma_neg_hi_mont, to_pinv;
  // Byte matrix of the tensor-core form (scale.cu), with its padded width;
  // empty when that form does not apply.
  DevBuf tc_mat;
  uint32_t tc_kp = 0;
  RnsScalerD(const Context& from, const Context& to, const BigUint& num, const BigUint& den);

 private:
  void build_tc_matrix();
};

// rq::Scaler (fhe-math/src/rq/scaler.rs:17-23).
struct Scaler {
  std::shared_ptr<Context> from, to;
  size_t number_common_moduli = 0;
  BigUint num, den;
  std::unique_ptr<RnsScalerD> rns;
  Scaler(std::shared_ptr<Context> from, std::shared_ptr<Context> to, const BigUint& num, const BigUint& den);
  bool is_one() const { return rns->host.is_one; }
};

// ---- operations on contexts (ops.cu) ----
void ntt_forward(const Context& ctx, PolyRef src, PolyRef dst, uint64_t polys, bool lazy, cudaStream_t st);
void ntt_backward(const Context& ctx, PolyRef src, PolyRef dst, uint64_t polys, cudaStream_t st);
void poly_op(const Context& ctx, int op, PolyRef a, PolyRef b, PolyRef out, uint64_t polys, cudaStream_t st);
// Representation::NttShoup (rq/mod.rs:37-47, 209-223): the Shoup plane of
// Ntt values, and the product of MulAssign<&Poly<NttShoup>> (rq/ops.rs:208-245).
void poly_compute_shoup(const Context& ctx, PolyRef a, PolyRef out, uint64_t polys, cudaStream_t st);
void poly_mul_shoup(const Context& ctx, PolyRef a, PolyRef b, PolyRef bs, PolyRef out, uint64_t polys,
                    cudaStream_t st);
constexpr size_t kMaxScalarLimbs = 64;
void poly_scalar_mul(const Context& ctx, const BigUint& scalar, PolyRef in, PolyRef out, uint64_t polys,
                     cudaStream_t st);
void poly_substitute(const Context& ctx, uint64_t exponent, bool ntt, PolyRef in, PolyRef out, uint64_t polys,
                     cudaStream_t st);
// Power-basis switch-down: in [L] limbs -> out [L-1] limbs.
void poly_switch_down_pb(const Context& ctx, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st);
// NTT switch-down: `in` is overwritten (it holds the power basis afterwards).
void poly_switch_down_ntt(const Context& ctx, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st);
// RnsScaler::scale over all coefficients: `in` power basis [from_len] limbs,
// `out` limbs k = 0..out_len-1 receive target modulus start + k.
// The strided last stages of a two-pass inverse NTT left to the consumer:
// `s1` stages of the source context (`primes`, one DevPrime per source
// limb), final scale N^-1 * 2^64 when `mont` (Montgomery products), else N^-1.
struct InverseTop {
  uint32_t s1;
  uint32_t mont;
  const DevPrime* primes;
};
// The strided first stages of two-pass forward NTTs applied by their
// producer, the RNS scaler: `s1` stages. Polynomials with poly % period <
// take (period 0: all) get them over their own output limbs (`primes`, one
// per output limb). With `digit_primes` set, the other polynomials are the c2
// of products: their output limb d is lifted into every key modulus j
// (reduced first unless `digit_raw`), given the stages there and written to
// digits.at((poly / period) * out_len + d, j).
struct ForwardTop {
  uint32_t s1;
  const DevPrime* primes;
  uint32_t period = 0, take = 1;
  const DevPrime* digit_primes = nullptr;
  uint32_t digit_limbs = 0, digit_raw = 0;
  PolyRef digits{};
};
// top != nullptr: `in` is the block pass of such a transform, and the scaler
// applies its last stages while loading (only where rns_scale_takes_top).
// fwd != nullptr (with top, the same s1): the outputs are written after the
// first stages of the forward NTT that consumes them.
void rns_scale(const RnsScalerD& s, uint32_t logn, PolyRef in, PolyRef out, uint32_t start, uint32_t out_len,
               uint64_t polys, cudaStream_t st, const InverseTop* top = nullptr, const ForwardTop* fwd = nullptr);
// Whether exact RNS scalings run on the tensor cores (default on), and the
// count of that form's bounded waits that ran out since the process started.
bool rns_tc_enabled();
void set_rns_tc(bool on);
uint64_t rns_tc_wait_failures();
bool rns_scale_takes_top(const RnsScalerD& s, uint32_t logn, uint32_t out_len, uint32_t s1);
// Scaler::scale. `scratch` must hold polys * max(L_from, L_to) * N words.
void scaler_scale(const Scaler& s, bool ntt, PolyRef in, PolyRef out, uint64_t polys, uint64_t* scratch,
                  cudaStream_t st);

// ---- BFV (bfv.cu) ----

// Plaintext side of a parameter set (codec.cu, built on first use).
struct PlainSide {
  std::shared_ptr<Context> tctx;       // modulus t, for SIMD (null if t has no NTT of size N)
  DevBuf maps;                         // u32 [N] matrix_reps_index_map, then u32 [N] its inverse
  std::shared_ptr<Context> plain_ctx;  // parameters.rs:480-494
  std::vector<std::unique_ptr<Scaler>> dec;  // per level: cipher context -> plaintext context by t / Q
};

struct Params {
  size_t degree = 0;
  std::vector<uint64_t> moduli;
  uint64_t plaintext = 0;
  std::vector<std::shared_ptr<Context>> levels;  // level l: first L-l moduli
  Params(size_t degree, const std::vector<uint64_t>& moduli, uint64_t plaintext);
  size_t max_level() const { return moduli.size() - 1; }
  const std::shared_ptr<Context>& ctx(size_t level) const;
  const PlainSide& plain_side() const;

 private:
  mutable std::mutex plain_mu;
  mutable std::unique_ptr<PlainSide> plain;
};

// A secret key on the device: s in Ntt form over the level-0 context.
struct SecretKeyDev {
  const Params* par = nullptr;
  DevBuf s_ntt;  // [L][N]
};

// Scratch memory of an operation: either a buffer the workspace owns and
// grows on demand, or an external region (a slice of the serving arena) of
// fixed size.
struct Workspace {
  DevBuf buf;
  uint64_t* ext = nullptr;
  size_t ext_bytes = 0;
  void attach(uint64_t* p, size_t bytes) {
    ext = p;
    ext_bytes = bytes;
  }
  void reserve(size_t bytes) {
    if (ext) {
      if (bytes > ext_bytes) throw Error(FHEG_ERR_BUDGET, "operation scratch exceeds the reserved region");
      return;
    }
    buf.reserve(bytes);
  }
  uint64_t* base() const { return ext ? ext : buf.u64(); }
  uint64_t* take(size_t words, size_t* offset) {
    uint64_t* p = base() + *offset;
    *offset += (words + 31) & ~(size_t)31;
    return p;
  }
};

struct Ksk {
  const Params* par = nullptr;
  size_t ciphertext_level = 0, ksk_level = 0;
  std::shared_ptr<Context> ctx_ct, ctx_ksk;
  size_t count = 0;  // digits: the moduli of the ciphertext context, or the decomposition's digits
  // Keys of a single-modulus key context decompose the input in base
  // 2^log_base instead of by residues (key_switching_key.rs:63-89, 292-329);
  // 0 for RNS-digit keys.
  uint32_t log_base = 0;
  // The 32-byte seed c1 was expanded from, when the key was made from one
  // (key_switching_key.rs:27-28); its message then carries the seed again.
  std::vector<uint8_t> seed;
  // [2 parts][count][Lk][N] values (canonical, Ntt representation).
  DevBuf keys;
  mutable Workspace ws;  // scratch of relinearize / galois_relinearize
  // When the key context has more moduli than the ciphertext context (a key
  // at a lower level), the constants of the switch-downs that bring a key
  // switch's output from one to the other (rq/mod.rs:455-462 switch_down_to,
  // one rq/mod.rs:390-448 switch_down per dropped modulus q_m, m = Lk-1 down
  // to L): per step [q_m, inv[0..m), inv_shoup[0..m), half[0..m)] with
  // inv[i] = q_m^-1 mod q_i and half[i] = q_i - (floor(q_m / 2) mod q_i).
  DevBuf chain;
  uint64_t* values(int part) const { return keys.u64() + (size_t)part * count * ctx_ksk->L() * ctx_ksk->N(); }
  // Whether the key switch ends in the key context and needs the switch-down.
  bool switches_down() const { return ctx_ksk->L() > ctx_ct->L(); }
};

// ilog2(next_power_of_two(q)) (key_switching_key.rs:71, 302-308).
inline uint32_t log_modulus_of(uint64_t q) { return 64 - (uint32_t)__builtin_clzll(q - 1); }
// Fills k.chain (nothing when the key and ciphertext contexts are equal).
void ksk_build_switch_chain(Ksk& k);
// Words of the D scratch key_switch() needs for `batch` polynomials: the
// digit NTTs and, for keys that switch down, the key context's outputs and
// their switched-down power basis.
size_t key_switch_scratch_words(const Ksk& k, uint64_t batch);
// switch_down_to (rq/mod.rs:455-462) of `polys` power-basis polynomials from
// the key context of `k` (Lk limbs, `in`) to its ciphertext context (L limbs,
// `out`), all steps fused per coefficient.
void switch_down_chain(const Ksk& k, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st);


// Key switch of digits already in the power basis: (out0, out1) =
// (add0 + sum_i NTT(d_i) * k0_i, add1 + sum_i NTT(d_i) * k1_i) where add0/add1
// are optional Ntt polynomials (with an optional substitution gather on add0).
// D holds key_switch_scratch_words(k, batch) words. With a key below the
// ciphertext level the sums are switched down to the ciphertext context
// before the additions (out then has the ciphertext context's L limbs).
void key_switch(const Ksk& k, PolyRef digits, uint64_t batch, const uint64_t* add0, uint64_t add0_poly_stride,
                uint64_t add0_exponent, const uint64_t* add1, uint64_t add1_poly_stride, uint64_t* out,
                uint64_t out_poly_stride, uint64_t* D, cudaStream_t st);


struct Multiplicator {
  const Params* par = nullptr;
  size_t level = 0;
  std::shared_ptr<Context> base, mul;
  std::unique_ptr<Scaler> ext_lhs, ext_rhs, down;
  const Ksk* rk = nullptr;
  bool mod_switch = false;
  // NTT block sizes of the stages (0 = the process-wide plan): A inverse of
  // the operands, C forward of the extension limbs, D tensor + inverse, F
  // forward of digits and c0 / c1 (f_split: digits and c0 / c1 as two
  // launches instead of one when F runs single-pass).
  uint32_t plan_a = 0, plan_c = 0, plan_d = 0, plan_f = 0;
  bool f_split = false;
  bool tensor_split = false;  // D as a product kernel plus an in-place inverse NTT
  // Batches of at most small_count pairs run with small_plan (same layout:
  // A, C, D, F, F split, D split) when its block sizes are valid for the
  // degree: a few ciphertexts do not fill the GPU with whole-limb CTAs, and
  // 2^12-residue blocks cut the one-pair latency by about 30% on GB300.
  uint64_t small_count = 8;
  uint32_t small_plan[6] = {12, 12, 12, 12, 1, 0};
  Workspace ws;
  DevBuf staging;  // device copies for the host entry point
  // `marks` (optional, 8 events) are recorded on `st` at the stage
  // boundaries: before A, after A, B, C, D, E, F and at the end.
  void multiply(const uint64_t* lhs, const uint64_t* rhs, uint64_t* out, uint64_t count, cudaStream_t st,
                Workspace* scratch = nullptr, cudaEvent_t* marks = nullptr);
  // Bytes of scratch multiply() needs for `count` pairs.
  size_t scratch_bytes(uint64_t count) const;
  size_t out_parts() const { return rk ? 2 : 3; }
  size_t out_level() const { return mod_switch ? level + 1 : level; }
};

std::unique_ptr<Multiplicator> make_multiplicator(const Params& par, size_t level, const BigUint& lhs_n,
                                                  const BigUint& lhs_d, const BigUint& rhs_n, const BigUint& rhs_d,
                                                  const std::vector<uint64_t>& ext, const BigUint& post_n,
                                                  const BigUint& post_d);
std::unique_ptr<Multiplicator> make_default_multiplicator(const Ksk& rk);

void relinearize(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st);
void relinearize_scratch(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, uint64_t* digits,
                         uint64_t* D, cudaStream_t st);
void galois_relinearize(const Ksk& gk, uint64_t exponent, const uint64_t* ct, uint64_t* out, uint64_t count,
                        Workspace& ws, cudaStream_t st);
// Poly::random_from_seed for `count` 32-byte device seeds: polynomial b
// ([L][N], the same values in every representation) at out + b * stride.
void poly_random_from_seed(const Context& c, const uint8_t* seeds, uint64_t* out, uint64_t stride, uint64_t count,
                           Workspace& ws, cudaStream_t st);
// The seeds of c1[0 .. count) of a key-switching key with seed `seed` (32
// bytes): 32 * count bytes (key_switching_key.rs:108-123).
// sample_vec_cbd (fhe-util/src/lib.rs:22-55) of `count` vectors of n
// samples, vector b drawn from ChaCha8Rng::from_seed(seeds[b]) (seeded.cu).
void sample_cbd_from_seed(const uint8_t* seeds, size_t variance, size_t n, size_t count, int64_t* out,
                          cudaStream_t st);
std::vector<uint8_t> ksk_c1_seeds(const uint8_t* seed, size_t count);

// External product with an RGSW ciphertext held as one key of 2L digits per
// part (ksk0's digits, then ksk1's): ct [count][2][L][N] -> out, both Ntt.
void external_product(const Ksk& rgsw, const uint64_t* ct, uint64_t* out, uint64_t count, Workspace& ws,
                      cudaStream_t st);
// One rotation of a ragged batch: ciphertext `ct` ([2][L][N] at the key's
// ciphertext level) rotated by `exponent` with `key`, into `out`.
struct RotRequest {
  const Ksk* key;
  uint64_t exponent;
  const uint64_t* ct;
  uint64_t* out;
};
// Checks every request of a batch (shared parameters, key levels, odd
// exponents) and throws before any device work if one is invalid.
void validate_rot_requests(const Params& par, const RotRequest* req, size_t count);
void galois_relinearize_batch(const Params& par, const RotRequest* req, size_t count, Workspace& ws,
                              cudaStream_t st);
size_t galois_batch_scratch_bytes(const RotRequest* req, size_t count);
// The batch's tables built in `ws` and uploaded (complete on return); the
// returned call launches the batch on a stream, reading no host memory, so
// it can be recorded into a CUDA graph. Buffers and keys must outlive it.
std::function<void(cudaStream_t)> prepare_galois_batch(const Params& par, const RotRequest* req, size_t count,
                                                       Workspace& ws, cudaStream_t st);
void ciphertext_switch_down(const Params& par, size_t level, size_t parts, uint64_t* ct, uint64_t* out,
                            uint64_t count, cudaStream_t st);

// ---- wire format (serialize.cu) ----
size_t poly_serialized_bytes(const Context& c);
void poly_serialize(const Context& c, int representation, const uint64_t* polys, uint8_t* bytes, uint64_t count,
                    DevBuf& scratch, cudaStream_t st);
void poly_deserialize(const Context& c, int representation, const uint8_t* bytes, uint64_t* polys, uint64_t count,
                      cudaStream_t st);

// ---- compositions (compose.cu) ----
void dot_product_scalar(const Params& par, size_t level, size_t parts, const uint64_t* cts, const uint64_t* pts,
                        uint64_t count, uint64_t groups, uint64_t* out, cudaStream_t st);
void inner_sum(const Params& par, const Ksk* const* keys, const uint64_t* exponents, size_t nkeys,
               const uint64_t* ct, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st);
void expand(const Params& par, const Ksk* const* keys, const uint64_t* exponents, size_t nlevels, size_t size,
            const uint64_t* ct, uint64_t* out, Workspace& ws, cudaStream_t st);

// ---- plaintext side (codec.cu) ----
void plaintext_encode(const Params& par, size_t level, const uint64_t* values, bool simd, uint64_t* pt_ntt,
                      uint64_t count, Workspace& ws, cudaStream_t st);
void ciphertext_mul_plain(const Params& par, size_t level, size_t parts, const uint64_t* ct, const uint64_t* pt,
                          bool pt_per_ct, uint64_t* out, uint64_t count, cudaStream_t st);
void encrypt(const SecretKeyDev& sk, size_t level, const uint64_t* values, bool simd, const uint64_t* a,
             const int64_t* e, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st);
size_t decrypt_scratch_bytes(const Params& par, size_t level, uint64_t count);
void decrypt(const SecretKeyDev& sk, size_t level, size_t parts, const uint64_t* ct, bool simd, uint64_t* values,
             uint64_t count, Workspace& ws, cudaStream_t st);

}  // namespace fheg
