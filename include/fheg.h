/*
 * fheg.h — C ABI of the GB300 RNS-BFV hot-path library (libfheg.so).
 *
 * This is the drop-in boundary for the ciphertext hot path of fhe.rs
 * (crates fhe-math and fhe). A Rust `-sys` crate binds these symbols and the
 * reference types forward to them; every entry point names the reference
 * interface it replaces (paths relative to the fhe.rs repository root).
 *
 * Conventions
 *  - All functions return an `int` status (FHEG_OK = 0). On failure a
 *    thread-local message is available from fheg_last_error().
 *  - Polynomials are limb-major arrays of u64 residues: a polynomial over a
 *    context with L moduli and degree N is `uint64_t[L][N]`, exactly the
 *    layout of `Poly::coefficients` (fhe-math/src/rq/mod.rs:124-132). A batch
 *    of `count` polynomials is `uint64_t[count][L][N]`; a batch of
 *    ciphertexts with `parts` polynomials each is `uint64_t[count][parts][L][N]`.
 *    A call takes at most 2^24 items (counts above return
 *    FHEG_ERR_INVALID_ARGUMENT).
 *  - `d_` pointers are device pointers (any CUDA allocation on the current
 *    device); `h_` pointers are host pointers. `stream` is a `cudaStream_t`
 *    (NULL = the legacy default stream).
 *  - Representations follow `rq::Representation`
 *    (fhe-math/src/rq/mod.rs:37-47): 0 = PowerBasis, 1 = Ntt, 2 = NttShoup.
 *    An NttShoup polynomial is its Ntt values plus, where an operation reads
 *    it, a second array of the same shape holding the Shoup plane
 *    (`coefficients_shoup`, rq/mod.rs:209-223; fheg_poly_compute_shoup).
 *  - Handles are opaque and thread-compatible: a handle may be used from
 *    several threads as long as calls on the same multiplicator or server are
 *    not concurrent.
 *  - Big integers (scaling factors) are little-endian arrays of u64 words.
 */
#ifndef FHEG_H
#define FHEG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define FHEG_EXTERN extern "C"
#else
#define FHEG_EXTERN extern
#endif
#define FHEG_API FHEG_EXTERN __attribute__((visibility("default")))

/* Status codes, mirroring the error kinds of fhe_math::Error
 * (fhe-math/src/errors.rs:9-40) and fhe::Error (fhe/src/errors.rs:15-129). */
enum fheg_status {
  FHEG_OK = 0,
  FHEG_ERR_INVALID_ARGUMENT = 1,   /* malformed sizes, null pointers */
  FHEG_ERR_INVALID_MODULUS = 2,    /* fhe_math::Error::InvalidModulus */
  FHEG_ERR_NTT_UNSUPPORTED = 3,    /* "Impossible to construct a Ntt operator" */
  FHEG_ERR_INVALID_CONTEXT = 4,    /* fhe_math::Error::InvalidContext / wrong poly context */
  FHEG_ERR_INVALID_LEVEL = 5,      /* fhe::Error::InvalidLevel */
  FHEG_ERR_KEY_MISMATCH = 6,       /* key / ciphertext level or context mismatch */
  FHEG_ERR_WRONG_PARTS = 7,        /* ciphertext has the wrong number of parts */
  FHEG_ERR_NO_MORE_CONTEXT = 8,    /* fhe_math::Error::NoMoreContext */
  FHEG_ERR_BUDGET = 9,             /* device memory budget exhausted */
  FHEG_ERR_CUDA = 10,              /* CUDA runtime error */
  FHEG_ERR_TIMEOUT = 11,           /* bounded wait expired */
  FHEG_ERR_UNSUPPORTED = 12,       /* valid request outside this library's scope */
  FHEG_ERR_INTERNAL = 13
};

typedef struct fheg_context fheg_context;
typedef struct fheg_scaler fheg_scaler;
typedef struct fheg_params fheg_params;
typedef struct fheg_ksk fheg_ksk;
typedef struct fheg_multiplicator fheg_multiplicator;
typedef struct fheg_graph fheg_graph;

/* ------------------------------------------------------------------------ */
/* Library                                                                    */

FHEG_API const char* fheg_version(void);
FHEG_API const char* fheg_status_string(int status);
/* Message of the last failed call on this thread ("" if none). */
FHEG_API const char* fheg_last_error(void);
/* Number of kernels this library has launched in this process (all devices).
 * Used by benchmarks to report how many of the library's kernels ran. */
FHEG_API uint64_t fheg_kernel_launch_count(void);
/* No counterpart in the reference: integer-throughput probes giving the
 * ceilings the NTT and RNS kernels are compared with. One launch of `blocks`
 * CTAs of 256 threads, each running `iters` iterations of 8 independent
 * register-resident chains of: kind 0 a 32-bit multiply-add (low half),
 * 1 a 32 x 32 -> 64-bit multiply-add, 2 a 32-bit multiply-add (high half),
 * 3 a 32-bit addition, 4 the NTT's Harvey forward butterfly (62-bit prime,
 * Shoup twiddle), 5 its Gentleman-Sande inverse butterfly. One word per
 * thread is written to d_sink (blocks * 256 words); *ops receives the
 * thread-level operations of the launch (time it on `stream`). */
FHEG_API int fheg_intpeak(int kind, size_t blocks, uint32_t iters, uint64_t* d_sink, void* stream, double* ops);

/* Device memory for callers without their own CUDA bindings (a Rust -sys
 * crate): plain cudaMalloc / cudaFree and stream-ordered copies. The copy to
 * the host returns after the copy completes. */
FHEG_API int fheg_device_alloc(size_t bytes, void** out);
FHEG_API int fheg_device_free(void* ptr);
FHEG_API int fheg_copy_to_device(void* d_dst, const void* h_src, size_t bytes, void* stream);
FHEG_API int fheg_copy_to_host(void* h_dst, const void* d_src, size_t bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Host-only number theory (no device work).                                  */

/* fhe-math/src/zq/primes.rs:30-59 `generate_prime`. *out = 0 when none. */
FHEG_API int fheg_generate_prime(uint32_t num_bits, uint64_t modulo, uint64_t upper_bound, uint64_t* out);
/* fhe-math/src/ntt/mod.rs:19-23 `supports_ntt`: 1 if p is prime and p = 1 mod 2n. */
FHEG_API int fheg_supports_ntt(uint64_t p, size_t n);
/* The default 2n-th root used by `NttOperator::new`
 * (fhe-math/src/ntt/native.rs:320-336). */
FHEG_API int fheg_ntt_default_root(uint64_t p, size_t n, uint64_t* out_root);
/* Host copy of the twiddle tables `NttOperator::new` builds
 * (fhe-math/src/ntt/native.rs:35-73): four arrays of n words each, and
 * size_inv / size_inv_shoup in out_size_inv[0..2]. root = 0 selects the
 * default root. */
FHEG_API int fheg_ntt_tables_host(uint64_t p, size_t n, uint64_t root, uint64_t* omegas,
                                  uint64_t* omegas_shoup, uint64_t* zetas_inv,
                                  uint64_t* zetas_inv_shoup, uint64_t* out_size_inv);
/* Host copy of the RnsScaler constants (fhe-math/src/rns/scaler.rs:79-175)
 * for the scaling from `from_moduli` to `to_moduli` by num/den. Output layout:
 *   out[0] = theta_garner_shift, out[1] = is_one,
 *   out[2..5] = theta_gamma (lo, hi, sign),
 *   then to_len gamma, to_len gamma_shoup,
 *   then to_len*from_len omega, to_len*from_len omega_shoup (row = target modulus),
 *   then from_len theta_omega_lo, from_len theta_omega_hi, from_len theta_omega_sign,
 *   then from_len theta_garner_lo, from_len theta_garner_hi.
 * `out_words` must be at least 5 + 2*to + 2*to*from + 5*from. */
FHEG_API int fheg_rns_scaler_constants_host(const uint64_t* from_moduli, size_t from_len,
                                            const uint64_t* to_moduli, size_t to_len,
                                            const uint64_t* num, size_t num_words,
                                            const uint64_t* den, size_t den_words,
                                            uint64_t* out, size_t out_words);

/* ------------------------------------------------------------------------ */
/* Ring contexts and polynomial operations (fhe-math `rq`, `ntt`, `rns`).     */

/* rq::Context::new (fhe-math/src/rq/context.rs:42-93). Uploads the NTT tables
 * of every modulus to the current device. `roots` (nullable) injects the 2N-th
 * root of each modulus, e.g. the root a caller's own `NttOperator` picked. */
FHEG_API int fheg_context_create(const uint64_t* moduli, size_t num_moduli, size_t degree,
                                 const uint64_t* roots, fheg_context** out);
FHEG_API void fheg_context_destroy(fheg_context* ctx);
FHEG_API size_t fheg_context_num_moduli(const fheg_context* ctx);
FHEG_API size_t fheg_context_degree(const fheg_context* ctx);

/* NttOperator::forward / forward_vt_lazy / backward
 * (fhe-math/src/ntt/native.rs:77-233) applied to every limb of `count`
 * polynomials in place: `Poly::into_ntt` / `into_power_basis`
 * (fhe-math/src/rq/mod.rs:294-313, 488-579). lazy = 1 leaves forward outputs
 * in [0, 4p) like `forward_vt_lazy`; otherwise outputs are reduced. */
FHEG_API int fheg_ntt_forward(const fheg_context* ctx, uint64_t* d_polys, size_t count, int lazy,
                              void* stream);
FHEG_API int fheg_ntt_backward(const fheg_context* ctx, uint64_t* d_polys, size_t count, void* stream);

/* NTT plan (no counterpart in the reference: it only changes how the GPU
 * schedules a transform, never its result). Transforms of 2^logn residues run
 * as one block (block_logn == logn, logn <= 14) or as a strided pass over the
 * first / last logn - block_logn stages plus blocks of 2^block_logn
 * (block_logn in 12..14, logn - block_logn <= 4). The plan is process-wide. */
FHEG_API int fheg_ntt_plan_set(uint32_t logn, uint32_t block_logn);
FHEG_API int fheg_ntt_plan_get(uint32_t logn, uint32_t* block_logn);
/* Whether NTT kernels hint the next CTA's input rows into L2 while they
 * work (off by default; schedules only). */
FHEG_API int fheg_ntt_prefetch_set(int on);
/* Cluster mode of a two-pass plan with 2^12-residue blocks (logn 13..16): the
 * transform runs as one pass on clusters of 2^(logn - 12) CTAs that exchange
 * the strided stages through distributed shared memory instead of a second
 * pass over device memory (GPUs that cannot run the cluster size fall back
 * to two passes). Schedules only; process-wide per logn. */
FHEG_API int fheg_ntt_cluster_set(uint32_t logn, int on);
FHEG_API int fheg_ntt_cluster_get(uint32_t logn, int* on);
/* Tensor-core form of the exact RNS scalings (rns/scaler.rs:249-352 through
 * RnsScaler::scale; no separate counterpart in the reference): for 12 to 32
 * source moduli and odd target moduli above 2^20, the products of the
 * residues with the scaler's constants run as byte-sliced FP16 matrix
 * products on tcgen05 (exact: every column sum stays below 2^24), and the
 * carries, rounding and reductions on the CUDA cores. On by default;
 * results are identical either way. Process-wide. */
FHEG_API int fheg_rns_tensor_set(int on);
FHEG_API int fheg_rns_tensor_get(int* on);
/* Number of bounded waits of the tensor-core scaler (operand copy, MMA
 * completion) that ran out since the library was loaded on the current
 * device; non-zero means some outputs of those launches are not valid. */
FHEG_API int fheg_rns_tensor_wait_failures(uint64_t* count);
/* Times every valid plan for the context's degree on `count` scratch
 * polynomials (forward + inverse), cluster mode included, installs the
 * fastest and returns its block size (fheg_ntt_cluster_get tells the mode). */
FHEG_API int fheg_ntt_autotune(const fheg_context* ctx, size_t count, void* stream, uint32_t* block_logn);

/* Coefficient-wise ring operations (fhe-math/src/rq/ops.rs:10-418):
 * op 0 = add, 1 = sub, 2 = mul (both Ntt, `MulAssign<&Poly<Ntt>>`),
 * 3 = neg (b ignored). d_out may alias d_a. */
FHEG_API int fheg_poly_op(const fheg_context* ctx, int op, const uint64_t* d_a, const uint64_t* d_b,
                          uint64_t* d_out, size_t count, void* stream);

/* The coefficient payload of the reference's `Rq` message
 * (fhe-math/src/rq/convert.rs:17-93): the power-basis coefficients of every
 * limb bit-packed little-endian with bitlen(q_j - 1) bits each
 * (zq/mod.rs:783-793, fhe-util/src/lib.rs:57-135), limbs concatenated.
 * representations 1 (Ntt) and 2 (NttShoup, values only) go through the power
 * basis as the reference does.
 * d_bytes holds count * fheg_poly_serialized_size bytes. Unpacked values are
 * reduced modulo their limb's modulus. The protobuf framing (representation,
 * degree, the bytes field) stays with the caller. */
FHEG_API int fheg_poly_serialized_size(const fheg_context* ctx, size_t* bytes);
FHEG_API int fheg_poly_serialize(const fheg_context* ctx, int representation, const uint64_t* d_polys,
                                 uint8_t* d_bytes, size_t count, void* stream);
FHEG_API int fheg_poly_deserialize(const fheg_context* ctx, int representation, const uint8_t* d_bytes,
                                   uint64_t* d_polys, size_t count, void* stream);

/* Poly::compute_coefficients_shoup (fhe-math/src/rq/mod.rs:209-223, the
 * conversion to NttShoup): d_shoup = floor(d_polys * 2^64 / q_j) for every
 * canonical residue. */
FHEG_API int fheg_poly_compute_shoup(const fheg_context* ctx, const uint64_t* d_polys, uint64_t* d_shoup,
                                     size_t count, void* stream);
/* MulAssign<&Poly<NttShoup>> for Poly<Ntt> (fhe-math/src/rq/ops.rs:208-245):
 * d_out = d_a * d_b coefficient-wise through d_b's Shoup plane, reduced.
 * d_out may alias d_a. */
FHEG_API int fheg_poly_mul_shoup(const fheg_context* ctx, const uint64_t* d_a, const uint64_t* d_b,
                                 const uint64_t* d_b_shoup, uint64_t* d_out, size_t count, void* stream);

/* MulAssign<&BigUint> for Poly (fhe-math/src/rq/ops.rs:297-352): every limb
 * times scalar mod q_j (scalar: little-endian u64 words), in either
 * representation. d_out may alias d_in. */
FHEG_API int fheg_poly_scalar_mul(const fheg_context* ctx, const uint64_t* scalar, size_t scalar_words,
                                  const uint64_t* d_in, uint64_t* d_out, size_t count, void* stream);

/* Poly::substitute (fhe-math/src/rq/mod.rs:319-369) for an odd exponent,
 * in Ntt (representation 1) or PowerBasis (0); NttShoup (2) permutes the
 * values as Ntt does (recompute the Shoup plane of the result with
 * fheg_poly_compute_shoup, rq/mod.rs:336-339). d_out must not alias d_in. */
FHEG_API int fheg_poly_substitute(const fheg_context* ctx, size_t exponent, int representation,
                                  const uint64_t* d_in, uint64_t* d_out, size_t count, void* stream);

/* Poly::switch_down (fhe-math/src/rq/mod.rs:390-448): drops the last modulus
 * with rounding. d_in is [count][L][N], d_out is [count][L-1][N]. In Ntt
 * representation the polynomial goes through the power basis like
 * `Ciphertext::switch_down` (fhe/src/bfv/ciphertext.rs:86-97). d_in is used as
 * scratch and is overwritten. */
FHEG_API int fheg_poly_switch_down(const fheg_context* ctx, int representation, uint64_t* d_in,
                                   uint64_t* d_out, size_t count, void* stream);

/* rq::Scaler::new (fhe-math/src/rq/scaler.rs:27-49) with the scaling factor
 * num/den (`ScalingFactor::new`, fhe-math/src/rns/scaler.rs:29-36). */
FHEG_API int fheg_scaler_create(const fheg_context* from, const fheg_context* to, const uint64_t* num,
                                size_t num_words, const uint64_t* den, size_t den_words,
                                fheg_scaler** out);
FHEG_API void fheg_scaler_destroy(fheg_scaler* s);
/* Poly::scale / Scaler::scale (fhe-math/src/rq/scaler.rs:52-126):
 * d_in [count][L_from][N] -> d_out [count][L_to][N] in the same
 * representation. d_in is not modified. */
FHEG_API int fheg_scaler_scale(const fheg_scaler* s, int representation, const uint64_t* d_in,
                               uint64_t* d_out, size_t count, void* stream);

/* Poly::random_from_seed (fhe-math/src/rq/mod.rs:239-257) for `count`
 * 32-byte seeds d_seeds [count][32] (device): polynomial b ([L][N], uniform
 * residues; the same values serve every representation) is written at
 * d_out + b * poly_stride words (poly_stride 0 = L*N; 2*L*N writes the c1 of
 * [count][2][L][N] ciphertexts, as a seeded Ciphertext is read,
 * fhe/src/bfv/ciphertext.rs:220-237). SHA-256 of the seed keys ChaCha8; each
 * limb takes N samples of Uniform[0, q_j) in turn. Calls on the same context
 * must not overlap (shared scratch). */
FHEG_API int fheg_poly_random_from_seed(const fheg_context* ctx, const uint8_t* d_seeds, uint64_t* d_out,
                                        size_t poly_stride, size_t count, void* stream);

/* sample_vec_cbd (fhe-util/src/lib.rs:22-55): d_out [count][n] signed
 * samples of the centered binomial distribution of `variance` (1..16), vector
 * b drawn from the next_u64 stream of ChaCha8Rng::from_seed(d_seeds[b])
 * (d_seeds [count][32] bytes on the device). With the seed of the caller's
 * ChaCha8Rng these are the errors of Poly::small (rq/mod.rs:262-284), the e
 * that SecretKey::try_encrypt (secret_key.rs:102-138) draws and that
 * fheg_encrypt takes. */
FHEG_API int fheg_sample_cbd_from_seed(const uint8_t* d_seeds, size_t variance, size_t n, size_t count,
                                       int64_t* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* BFV (crate fhe).                                                           */

/* BfvParametersBuilder::build (fhe/src/bfv/parameters.rs:431-641) for the
 * parts the hot path needs: the context chain, one context per level
 * (level l keeps the first L-l moduli). */
FHEG_API int fheg_params_create(size_t degree, const uint64_t* moduli, size_t num_moduli,
                                uint64_t plaintext, fheg_params** out);
FHEG_API void fheg_params_destroy(fheg_params* par);
/* BfvParameters::context_at_level (parameters.rs:155-177). The context is
 * owned by the parameters. */
FHEG_API int fheg_params_context_at_level(const fheg_params* par, size_t level, const fheg_context** out);
FHEG_API size_t fheg_params_max_level(const fheg_params* par);

/* A key-switching key resident on the device: `KeySwitchingKey`
 * (fhe/src/bfv/keys/key_switching_key.rs:21-45), RNS-digit form. h_c0 and
 * h_c1 hold the `c0[i]` / `c1[i]` polynomials (Ntt values, canonical) as
 * [count][L_ksk][N] host arrays with count = number of ciphertext moduli;
 * the Shoup companions are computed here. */
FHEG_API int fheg_ksk_create(const fheg_params* par, size_t ciphertext_level, size_t ksk_level,
                             const uint64_t* h_c0, const uint64_t* h_c1, size_t count, fheg_ksk** out);
/* A key-switching key from its c0[i] polynomials and the 32-byte seed the
 * reference stores instead of c1 (`KeySwitchingKey::seed`,
 * key_switching_key.rs:67-68; c1 regenerated as generate_c1 does,
 * key_switching_key.rs:108-123, 383-406): c1[i] = Poly::random_from_seed of
 * the i-th 32 bytes of ChaCha8Rng::from_seed(seed), expanded on the device. */
FHEG_API int fheg_ksk_create_seeded(const fheg_params* par, size_t ciphertext_level, size_t ksk_level,
                                    const uint64_t* h_c0, const uint8_t* seed, size_t count, fheg_ksk** out);
FHEG_API void fheg_ksk_destroy(fheg_ksk* k);

/* RelinearizationKey::relinearizes (fhe/src/bfv/keys/relinearization_key.rs:71-98):
 * d_ct3 [count][3][L][N] (Ntt) -> d_out [count][2][L][N] (Ntt). A key whose
 * level is below the ciphertext level (more moduli) key-switches in its own
 * context and switches the result down to the ciphertext context before the
 * additions (relinearization_key.rs:84-92); the same holds for Galois keys
 * (galois_key.rs:113-120) and for the relinearization of the Multiplicator
 * (fhe/src/bfv/ops/mul.rs:199-206). */
FHEG_API int fheg_relinearize(const fheg_ksk* rk, const uint64_t* d_ct3, uint64_t* d_out, size_t count,
                              void* stream);

/* GaloisKey::relinearize / relinearize_into (fhe/src/bfv/keys/galois_key.rs:63-124),
 * reached through EvaluationKey::rotates_columns_by (exponent 3^i mod 2N) and
 * rotates_rows (exponent 2N-1) (fhe/src/bfv/keys/evaluation_key.rs:92-131).
 * d_ct [count][2][L][N] (Ntt) -> d_out [count][2][L][N] (Ntt). */
FHEG_API int fheg_galois_relinearize(const fheg_ksk* gk, size_t exponent, const uint64_t* d_ct,
                                     uint64_t* d_out, size_t count, void* stream);

/* A ragged batch of rotations: ciphertext b (at its key's ciphertext level,
 * [2][L_b][N] Ntt) is rotated with keys[b] by exponents[b] into d_outs[b],
 * exactly as GaloisKey::relinearize_into (galois_key.rs:90-124) would one at a
 * time (EvaluationKey::rotates_columns_by / rotates_rows,
 * evaluation_key.rs:92-131). Ciphertexts may sit at different levels; all keys
 * must come from `par`. One launch per stage covers the whole batch; from 16
 * requests the two halves run concurrently, the second on a stream of the
 * parameters' that forks from and joins `stream`. Calls on the same
 * parameters must not run concurrently (shared scratch). */
FHEG_API int fheg_galois_relinearize_batch(const fheg_params* par, const fheg_ksk* const* keys,
                                           const size_t* exponents, const uint64_t* const* d_cts,
                                           uint64_t* const* d_outs, size_t count, void* stream);
/* No counterpart in the reference: the same ragged batch recorded once as a
 * CUDA graph (fheg_graph_launch replays it on whatever the ciphertext buffers
 * hold then; fheg_graph_destroy frees it). Its tables and scratch belong to
 * the graph; the keys and buffers must outlive it. Runs the batch once while
 * recording (the outputs are written). */
FHEG_API int fheg_galois_relinearize_batch_capture(const fheg_params* par, const fheg_ksk* const* keys,
                                                   const size_t* exponents, const uint64_t* const* d_cts,
                                                   uint64_t* const* d_outs, size_t count, fheg_graph** out);

/* Ciphertext::switch_down (fhe/src/bfv/ciphertext.rs:86-97) for ciphertexts
 * at `level` with `parts` polynomials: d_ct [count][parts][L][N] ->
 * d_out [count][parts][L-1][N]. d_ct is used as scratch. */
FHEG_API int fheg_ciphertext_switch_down(const fheg_params* par, size_t level, size_t parts,
                                         uint64_t* d_ct, uint64_t* d_out, size_t count, void* stream);

/* Ciphertext::switch_to_level (fhe/src/bfv/ciphertext.rs:100-119): repeated
 * switch_down from `level` to `target_level` (level <= target_level <=
 * max_level, else FHEG_ERR_INVALID_LEVEL). d_ct [count][parts][L][N] is used as
 * scratch; d_out receives [count][parts][L'][N] at the target level. The
 * intermediate levels use the parameters' scratch region, so calls on the same
 * parameters must not overlap. */
FHEG_API int fheg_ciphertext_switch_to_level(const fheg_params* par, size_t level, size_t target_level,
                                             size_t parts, uint64_t* d_ct, uint64_t* d_out, size_t count,
                                             void* stream);

/* Add<&Ciphertext> (fhe/src/bfv/ops/mod.rs:15-43). */
FHEG_API int fheg_ciphertext_add(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_a,
                                 const uint64_t* d_b, uint64_t* d_out, size_t count, void* stream);

/* Multiplicator::default(&rk) (fhe/src/bfv/ops/mul.rs:101-130): extension
 * basis generated as the reference does, relinearization enabled. */
FHEG_API int fheg_multiplicator_create_default(const fheg_ksk* rk, fheg_multiplicator** out);
/* Multiplicator::new_leveled (fhe/src/bfv/ops/mul.rs:56-98) with explicit
 * scaling factors and extended basis (whose first moduli must be the level's
 * moduli when a factor is one). */
FHEG_API int fheg_multiplicator_create(const fheg_params* par, size_t level, const uint64_t* lhs_num,
                                       size_t lhs_num_words, const uint64_t* lhs_den, size_t lhs_den_words,
                                       const uint64_t* rhs_num, size_t rhs_num_words, const uint64_t* rhs_den,
                                       size_t rhs_den_words, const uint64_t* extended_basis,
                                       size_t extended_len, const uint64_t* post_num, size_t post_num_words,
                                       const uint64_t* post_den, size_t post_den_words,
                                       fheg_multiplicator** out);
FHEG_API void fheg_multiplicator_destroy(fheg_multiplicator* m);
/* Multiplicator::enable_relinearization / enable_mod_switching (mul.rs:133-155). */
FHEG_API int fheg_multiplicator_enable_relinearization(fheg_multiplicator* m, const fheg_ksk* rk);
FHEG_API int fheg_multiplicator_enable_mod_switching(fheg_multiplicator* m);
/* Shape of the product: parts (2 with relinearization, else 3) and level. */
FHEG_API int fheg_multiplicator_output_shape(const fheg_multiplicator* m, size_t* parts, size_t* level);
/* Multiplicator::multiply (fhe/src/bfv/ops/mul.rs:158-227), batched:
 * d_lhs, d_rhs [count][2][L][N] (Ntt) -> d_out [count][parts][L'][N].
 * From 32 pairs the two halves of the batch run concurrently, the second on
 * a stream of the multiplicator's that forks from and joins `stream`. */
FHEG_API int fheg_multiplicator_multiply(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                         uint64_t* d_out, size_t count, void* stream);
/* No counterpart in the reference: several batched multiplications issued
 * together, typically one per level of one parameter set (a batch of
 * ciphertexts at mixed levels, grouped by level): group g multiplies
 * counts[g] pairs d_lhs[g] x d_rhs[g] -> d_out[g] with mults[g] (layouts as
 * fheg_multiplicator_multiply at that multiplicator's level). Each group runs
 * on its multiplicator's own stream, forked from and joined back into
 * `stream`, so the groups' kernels overlap on the GPU. A multiplicator may
 * appear in one group only (merge its pairs into one batch). */
FHEG_API int fheg_multiply_groups(fheg_multiplicator* const* mults, const uint64_t* const* d_lhs,
                                  const uint64_t* const* d_rhs, uint64_t* const* d_out, const size_t* counts,
                                  size_t groups, void* stream);
/* Runs one multiplication with events at the stage boundaries and returns
 * the duration of each stage in ms[7]: A inverse NTT of the operands,
 * B basis extension, C forward NTT of the extension limbs, D tensor product
 * + inverse NTT, E t/Q scaling, F digit and c0 / c1 NTTs, G key inner product
 * (and the switch-down when enabled). No counterpart in the reference. */
FHEG_API int fheg_multiplicator_stage_times(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                            uint64_t* d_out, size_t count, void* stream, float* ms);
/* Per-stage NTT plans of a multiplicator (no counterpart in the reference:
 * schedules only, results are unchanged). plan[6] = block log2 of stage A
 * (inverse NTT of the operands), C (forward NTT of the extension limbs),
 * D (tensor product + inverse NTT), F (digit and c0 / c1 forward NTTs),
 * plan[4] = 1 to run F as two launches when it is single-pass, and plan[5] =
 * 1 to run the tensor product of D as its own kernel before the inverse NTT.
 * Block sizes follow fheg_ntt_plan_set's rules. */
FHEG_API int fheg_multiplicator_get_plan(const fheg_multiplicator* m, uint32_t* plan);
FHEG_API int fheg_multiplicator_set_plan(fheg_multiplicator* m, const uint32_t* plan);
/* Plan for small batches: multiplications of at most max_count pairs use
 * plan[6] instead (default: 8 pairs, blocks of 2^12 with F in two launches,
 * which cuts the one-pair latency by about 30% at N = 2^14). max_count = 0
 * turns it off. */
FHEG_API int fheg_multiplicator_set_small_plan(fheg_multiplicator* m, size_t max_count, const uint32_t* plan);
/* Times the multiplication of `count` pairs while varying one stage's plan
 * at a time, installs the fastest and returns it in plan[6] (may be NULL).
 * A count within the small-batch threshold tunes the small-batch plan. */
FHEG_API int fheg_multiplicator_autotune(fheg_multiplicator* m, size_t count, void* stream, uint32_t* plan);
/* Pipeline of fheg_multiplicator_multiply_host: `chunk` pairs per chunk
 * (0 = automatic: 4 when count >= 8, else the whole call) multiplied on
 * `streams` compute streams in turn (1..4, default 3), each with its own
 * scratch; the inputs and outputs cross the host link on two copy streams
 * of their own. Changes only the overlap of copies and compute, never the
 * results. No counterpart in the reference. */
FHEG_API int fheg_multiplicator_set_host_pipeline(fheg_multiplicator* m, size_t chunk, int streams);
/* Multiplicator::multiply end to end from host buffers (h_lhs, h_rhs
 * [count][2][L][N], h_out the output shape): copies the inputs to the
 * device, multiplies, and copies the product back before returning. */
FHEG_API int fheg_multiplicator_multiply_host(fheg_multiplicator* m, const uint64_t* h_lhs,
                                              const uint64_t* h_rhs, uint64_t* h_out, size_t count);

/* ------------------------------------------------------------------------ */
/* Allocation-free relinearization.                                           */

/* No counterpart in the reference: this entry point exists for callers of
 * this library that cannot let it allocate device memory, such as code
 * recording into a CUDA stream capture (cudaMalloc cannot be captured),
 * serving loops that must not stall on an allocation, and applications that
 * give all device memory to their own pool. It computes what
 * fheg_relinearize computes (d_ct3 [count][3][L][N] Ntt -> d_out
 * [count][2][L][N] Ntt) and calls no cudaMalloc / cudaFree: its scratch is a
 * fixed 16 MiB device array inside the library, which every GPU that loads the
 * library holds until the process exits. A call needs
 * 8 * count * L * N * (1 + L_ksk) bytes, plus 8 * count * N * 2 * (L_ksk + L)
 * for a key below the ciphertext level (each region rounded up to 256 bytes);
 * larger batches are rejected with FHEG_ERR_INVALID_ARGUMENT
 * (split them). The first call on a device looks the array's address up, so
 * make it before any stream capture. All calls share the array and it keeps
 * the last call's contents: calls whose work overlaps on the GPU (different
 * streams, or different threads without ordering) race on it. */
FHEG_API int fheg_relinearize_noalloc(const fheg_ksk* rk, const uint64_t* d_ct3, uint64_t* d_out, size_t count,
                                      void* stream);

/* ------------------------------------------------------------------------ */
/* Plaintext side: encoding, ciphertext x plaintext, decryption               */

typedef struct fheg_secret_key fheg_secret_key;

/* The Ntt polynomial a Plaintext carries (`poly_ntt`, plaintext_vec.rs:40-100)
 * for `count` vectors d_values [count][N] of values below t (pad with zeros):
 * simd != 0 scatters them by `matrix_reps_index_map` (parameters.rs:616-629)
 * and applies the inverse NTT mod t; the result is lifted into the context of
 * `level` and transformed: d_pt_ntt [count][L][N]. Uses the parameters'
 * scratch region (calls on the same parameters must not overlap). */
FHEG_API int fheg_plaintext_encode(const fheg_params* par, size_t level, const uint64_t* d_values, int simd,
                                   uint64_t* d_pt_ntt, size_t count, void* stream);

/* MulAssign<&Plaintext> for Ciphertext (fhe/src/bfv/ops/mod.rs:229-238):
 * every part of d_ct [count][parts][L][N] times the plaintext polynomial
 * (d_pt_ntt [L][N] shared, or [count][L][N] with pt_per_ciphertext != 0). */
FHEG_API int fheg_ciphertext_mul_plain(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_ct,
                                       const uint64_t* d_pt_ntt, int pt_per_ciphertext, uint64_t* d_out,
                                       size_t count, void* stream);

/* A secret key (SecretKey::coeffs, secret_key.rs:24-60: N signed
 * coefficients) resident on the device in Ntt form. */
FHEG_API int fheg_secret_key_create(const fheg_params* par, const int64_t* coeffs, fheg_secret_key** out);
FHEG_API void fheg_secret_key_destroy(fheg_secret_key* sk);

/* SecretKey::try_encrypt (secret_key.rs:102-138, 186-194) with its
 * randomness supplied by the caller: d_a [count][L][N] the uniform Ntt
 * polynomial a (Poly::random_from_seed in the reference), d_e [count][N] the
 * small error coefficients (Poly::small). d_values [count][N] (< t) are the
 * plaintext slots (simd != 0) or coefficients. d_ct [count][2][L][N] receives
 * (e - a s + m, a). Calls on the same key must not overlap. */
FHEG_API int fheg_encrypt(const fheg_secret_key* sk, size_t level, const uint64_t* d_values, int simd,
                          const uint64_t* d_a, const int64_t* d_e, uint64_t* d_ct, size_t count, void* stream);

/* SecretKey::try_decrypt (secret_key.rs:200-252) followed by decoding
 * (plaintext.rs:337-390): d_ct [count][parts][L][N] at `level` ->
 * d_values [count][N] mod t (simd != 0: slot order; 0: coefficient order).
 * Calls on the same key must not overlap (shared scratch). */
FHEG_API int fheg_decrypt(const fheg_secret_key* sk, size_t level, size_t parts, const uint64_t* d_ct, int simd,
                          uint64_t* d_values, size_t count, void* stream);

/* dot_product_scalar (fhe/src/bfv/ops/dot_product.rs:56-140) for `groups`
 * independent dot products over the same `count` plaintexts:
 * d_out[g] = sum_c d_cts[g][c] * d_pts[c], with d_cts
 * [groups][count][parts][L][N], d_pts [count][L][N] (Ntt polynomials of the
 * plaintexts, fheg_plaintext_encode) and d_out [groups][parts][L][N]. */
FHEG_API int fheg_dot_product_scalar(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_cts,
                                     const uint64_t* d_pts, size_t count, size_t groups, uint64_t* d_out,
                                     void* stream);

/* EvaluationKey::computes_inner_sum (fhe/src/bfv/keys/evaluation_key.rs:56-83)
 * on d_ct [count][2][L][N]: keys / exponents in the reference's order (column
 * rotations by 1, 2, 4, ... < N/2 as exponents 3^i mod 2N, then the row
 * rotation 2N - 1), all at the ciphertext's level. Uses the parameters'
 * scratch region (calls on the same parameters must not overlap). */
FHEG_API int fheg_inner_sum(const fheg_params* par, const fheg_ksk* const* keys, const size_t* exponents,
                            size_t nkeys, const uint64_t* d_ct, uint64_t* d_out, size_t count, void* stream);

/* EvaluationKey::expands (evaluation_key.rs:148-193): the oblivious expansion
 * of one ciphertext d_ct [2][L][N] into d_out [size][2][L][N]; keys[l] is the
 * Galois key of exponent (N >> l) + 1, for l < ceil(log2(size)) <= nlevels. */
FHEG_API int fheg_expand(const fheg_params* par, const fheg_ksk* const* keys, const size_t* exponents,
                         size_t nlevels, size_t size, const uint64_t* d_ct, uint64_t* d_out, void* stream);

/* RGSWCiphertext (fhe/src/bfv/rgsw_ciphertext.rs:19-24): the key-switching
 * keys ksk0 (of m) and ksk1 (of m s), both with ciphertext level = key level
 * = `level` (the reference rejects other levels, rgsw_ciphertext.rs:59-68).
 * h_ksk0_c0 .. h_ksk1_c1 are the keys' c0[i] / c1[i] polynomials as
 * [L][L][N] host arrays (Ntt values, canonical), L = moduli at `level`. */
typedef struct fheg_rgsw fheg_rgsw;
FHEG_API int fheg_rgsw_create(const fheg_params* par, size_t level, const uint64_t* h_ksk0_c0,
                              const uint64_t* h_ksk0_c1, const uint64_t* h_ksk1_c0, const uint64_t* h_ksk1_c1,
                              fheg_rgsw** out);
FHEG_API void fheg_rgsw_destroy(fheg_rgsw* rgsw);

/* Mul<&RGSWCiphertext> for &Ciphertext (rgsw_ciphertext.rs:123-160; the
 * product is commutative): the external product of every ciphertext of
 * d_ct [count][2][L][N] (Ntt, at the RGSW ciphertext's level) -> d_out
 * [count][2][L][N] (Ntt). Calls on the same RGSW ciphertext must not overlap
 * (shared scratch). */
FHEG_API int fheg_external_product(const fheg_rgsw* rgsw, const uint64_t* d_ct, uint64_t* d_out, size_t count,
                                   void* stream);

/* ------------------------------------------------------------------------ */
/* Ciphertext messages (bfv.proto `Ciphertext` holding rq.proto `Rq` parts,   */
/* encoded as the reference's prost encoding does: fields in tag order,       */
/* proto3 defaults left out).                                                 */

/* Bytes of one message from fheg_ciphertext_to_bytes: `parts` polynomials at
 * `level`; seeded != 0 when the last part is replaced by its 32-byte seed;
 * allow_variable_time is the Rq flag written for every part. */
FHEG_API int fheg_ciphertext_serialized_size(const fheg_params* par, size_t level, size_t parts, int seeded,
                                             int allow_variable_time, size_t* bytes);
/* Ciphertext::to_bytes (fhe/src/bfv/ciphertext.rs:164-191,
 * fhe-math/src/rq/convert.rs:17-42) for d_ct [count][parts][L][N] (Ntt):
 * h_out receives `count` messages of fheg_ciphertext_serialized_size bytes,
 * back to back. h_seeds (nullable) [count][32] are the seeds of the last
 * parts (Ciphertext::seed), written in place of those parts. Returns once
 * h_out is written. Uses the parameters' scratch region. */
FHEG_API int fheg_ciphertext_to_bytes(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_ct,
                                      size_t count, const uint8_t* h_seeds, int allow_variable_time,
                                      uint8_t* h_out, size_t out_capacity, void* stream);
/* Level, number of parts and seededness of one message, with the
 * reference's checks (ciphertext.rs:196-216: "Not enough polynomials" ->
 * FHEG_ERR_WRONG_PARTS, a level above the maximum -> FHEG_ERR_INVALID_LEVEL,
 * a seed of another length than 32 bytes). No device work. */
FHEG_API int fheg_ciphertext_peek(const fheg_params* par, const uint8_t* h_msg, size_t len, size_t* level,
                                  size_t* parts, int* seeded);
/* Ciphertext::from_bytes (ciphertext.rs:195-240, rq/convert.rs:44-135) for
 * `count` messages h_msgs[b] of lens[b] bytes that all decode to `level` and
 * `parts` and are all seeded or all unseeded (fheg_ciphertext_peek tells):
 * d_out [count][parts][L][N] (Ntt). Payloads are unpacked and transformed on
 * the device and seeded last parts expanded there (Poly::random_from_seed).
 * Rq errors: representation other than Ntt, degree not a multiple of 8 or
 * not the context's, payload of the wrong length -> FHEG_ERR_INVALID_ARGUMENT.
 * Returns once the messages may be freed. Uses the parameters' scratch. */
FHEG_API int fheg_ciphertext_from_bytes(const fheg_params* par, const uint8_t* const* h_msgs, const size_t* lens,
                                        size_t count, size_t level, size_t parts, uint64_t* d_out, void* stream);

/* KeySwitchingKey::from_bytes (fhe/src/bfv/keys/key_switching_key.rs:354-420)
 * of a serialized key: kind 0 a bare KeySwitchingKey message, 1 a
 * RelinearizationKey (relinearization_key.rs:109-127), 2 a GaloisKey
 * (galois_key.rs:127-149; *exponent receives its exponent, which must be
 * odd and below 2N). c0[i] and c1[i] are NttShoup Rq messages over the key
 * context; a key that carries its seed has its c1 expanded on the device
 * (generate_c1). Errors as the reference: wrong number of c0 / c1 values or
 * a seed of another length, a decomposition base (log_base != 0) with levels
 * that are not maximal -> FHEG_ERR_INVALID_ARGUMENT, levels above the
 * maximum -> FHEG_ERR_INVALID_LEVEL. A decomposition base names a
 * single-modulus key of ceil(log2 q / log_base) digits (key_switching_key.rs:
 * 360-372). The key's levels are returned in *ciphertext_level and
 * *ksk_level (each output nullable). */
FHEG_API int fheg_ksk_from_bytes(const fheg_params* par, const uint8_t* h_msg, size_t len, int kind,
                                 fheg_ksk** out, size_t* exponent, size_t* ciphertext_level, size_t* ksk_level);

/* KeySwitchingKey (kind 0), RelinearizationKey (1) and GaloisKey (2, with its
 * `exponent`) to_bytes (key_switching_key.rs:332-352,
 * relinearization_key.rs:109-115, 129-131, galois_key.rs:127-134) of a
 * device key: c0[i], then c1[i] or, for a key made from its seed, the seed,
 * as NttShoup Rq messages (payloads of the power basis of the values, with
 * allow_variable_time set, as the reference's keys carry it), then the
 * levels and the decomposition base; fields in prost's order. The message
 * goes to h_out (capacity `cap`); *len receives its length. h_out = NULL
 * asks for the length only. */
FHEG_API int fheg_ksk_to_bytes(const fheg_ksk* key, int kind, size_t exponent, uint8_t* h_out, size_t cap,
                               size_t* len);
/* EvaluationKey::to_bytes (fhe/src/bfv/keys/evaluation_key.rs:210-213,
 * 382-392): { repeated GaloisKey gk = 2; ciphertext_level = 3;
 * evaluation_key_level = 4 } with the `count` keys in the order given (the
 * reference iterates a hash map, so its order is unspecified). Every key must
 * be at the two levels (FHEG_ERR_KEY_MISMATCH). Output as fheg_ksk_to_bytes. */
FHEG_API int fheg_evaluation_key_to_bytes(const fheg_ksk* const* keys, const size_t* exponents, size_t count,
                                          size_t ciphertext_level, size_t evaluation_key_level, uint8_t* h_out,
                                          size_t cap, size_t* len);
/* EvaluationKey::from_bytes (evaluation_key.rs:216-228, 394-432): decodes
 * every Galois key of the message into keys[i] with its exponent in
 * exponents[i] (the caller destroys them); *count receives the number of keys
 * and the levels go to the nullable outputs. keys = NULL asks for the count
 * only; fewer than *count slots -> FHEG_ERR_INVALID_ARGUMENT. A key at other
 * levels than the message names fails as in the reference. */
FHEG_API int fheg_evaluation_key_from_bytes(const fheg_params* par, const uint8_t* h_msg, size_t len,
                                            fheg_ksk** keys, size_t* exponents, size_t cap, size_t* count,
                                            size_t* ciphertext_level, size_t* evaluation_key_level);

/* ------------------------------------------------------------------------ */
/* CUDA graphs                                                                */

/* Records Multiplicator::multiply for fixed device buffers (d_lhs, d_rhs:
 * [count][2][L][N], d_out: the multiplicator's output shape) into a CUDA
 * graph; each fheg_graph_launch replays the whole pipeline with one call.
 * The graph owns its scratch. It runs the multiplication once before
 * recording (so d_out is written). Batches of 32 pairs or more are recorded
 * as two independent branches of half the batch each, which the GPU runs
 * concurrently (the kernels of one branch fill the gaps of the other).
 * Destroy the graph before the multiplicator and its key. No counterpart in
 * the reference. */
FHEG_API int fheg_multiplicator_capture(fheg_multiplicator* m, const uint64_t* d_lhs, const uint64_t* d_rhs,
                                        uint64_t* d_out, size_t count, fheg_graph** out);
FHEG_API int fheg_graph_launch(const fheg_graph* g, void* stream);
/* Number of kernels one replay launches. */
FHEG_API int fheg_graph_kernel_count(const fheg_graph* g, uint64_t* kernels);
FHEG_API void fheg_graph_destroy(fheg_graph* g);

/* ------------------------------------------------------------------------ */
/* Serving runtime                                                            */

/* No counterpart in the reference (fhe.rs evaluates one operation per call on
 * the caller's thread). A server owns a fixed device-memory budget and a
 * scheduler thread that batches pending requests with the same operation and
 * parameters (rotations with any keys, exponents and levels batch together),
 * admits a batch when one of its streams is free and the batch's inputs,
 * outputs and scratch fit in the budget, and runs host->device copies, the
 * batched operation and device->host copies on that stream. Results are
 * bit-identical to the single-operation entry points. A request that does not
 * fit in the budget even alone completes with FHEG_ERR_BUDGET. */
typedef struct fheg_server fheg_server;

typedef struct fheg_server_config {
  size_t hbm_budget_bytes; /* device arena (inputs, outputs and scratch of running batches) */
  uint32_t streams;        /* batches in flight at once */
  uint32_t max_batch;      /* requests per batch */
} fheg_server_config;

enum fheg_server_op {
  FHEG_OP_MUL_RELIN = 0,   /* Multiplicator::multiply (fhe/src/bfv/ops/mul.rs:158-227) */
  FHEG_OP_ROTATE = 1,      /* GaloisKey::relinearize (fhe/src/bfv/keys/galois_key.rs:63-124) */
  FHEG_OP_ADD = 2,         /* Add<&Ciphertext> (fhe/src/bfv/ops/mod.rs:15-43) */
  FHEG_OP_SWITCH_DOWN = 3  /* Ciphertext::switch_down (fhe/src/bfv/ciphertext.rs:86-97) */
};

typedef struct fheg_request {
  int op;                          /* enum fheg_server_op */
  const fheg_params* par;
  const fheg_multiplicator* mult;  /* FHEG_OP_MUL_RELIN */
  const fheg_ksk* key;             /* FHEG_OP_ROTATE */
  size_t exponent;                 /* FHEG_OP_ROTATE */
  size_t level;                    /* FHEG_OP_ADD, FHEG_OP_SWITCH_DOWN */
  const uint64_t* in0;             /* host [2][L][N] */
  const uint64_t* in1;             /* host [2][L][N] (MUL_RELIN, ADD) */
  uint64_t* out;                   /* host, the shape of the operation's result */
} fheg_request;

FHEG_API int fheg_server_create(const fheg_server_config* cfg, fheg_server** out);
/* Finishes every submitted request, then stops the scheduler. */
FHEG_API void fheg_server_destroy(fheg_server* s);
/* Validates and queues a request; host buffers must stay valid until it completes. */
FHEG_API int fheg_server_submit(fheg_server* s, const fheg_request* req, uint64_t* id);
/* Waits at most timeout_ms for the request; returns its status, or
 * FHEG_ERR_TIMEOUT when it has not completed yet. */
FHEG_API int fheg_server_wait(fheg_server* s, uint64_t id, uint32_t timeout_ms);
/* Host steady-clock times (ns) of submission, batch start and completion. */
FHEG_API int fheg_server_request_times(fheg_server* s, uint64_t id, int64_t* submit_ns, int64_t* start_ns,
                                       int64_t* done_ns);
/* Forgets a completed request. */
FHEG_API int fheg_server_release(fheg_server* s, uint64_t id);
FHEG_API int fheg_server_stats(fheg_server* s, uint64_t* submitted, uint64_t* completed, uint64_t* batches,
                               size_t* peak_bytes);

#endif /* FHEG_H */
