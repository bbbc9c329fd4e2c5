// Operations composed of the key-switching path: the inner sum and the
// oblivious expansion of EvaluationKey, and the ciphertext-plaintext dot
// product (fhe/src/bfv/keys/evaluation_key.rs:56-193,
// fhe/src/bfv/ops/dot_product.rs:56-140).

#include <vector>

#include "fheg.h"
#include "handles.hpp"
#include "abi_call.hpp"
#include "lib.hpp"

namespace fheg {

namespace {

unsigned nblk(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

// out[g][k][j][i] = sum_c ct[g][c][k][j][i] * pt[c][j][i] mod q_j: exact
// 128-bit sums of products below 2^124, reduced every 15 terms and at the end
// (the reference accumulates in u128 and reduces once; both give the
// canonical residue).
__global__ void k_dot_product(const DevPrime* primes, const uint64_t* ct, const uint64_t* pt, uint64_t* out,
                              uint32_t count, uint32_t parts, uint32_t limbs, uint32_t logn, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t row = row_of(gid, logn);  // (g, k, j)
  const uint32_t j = row % limbs;
  const uint32_t k = (row / limbs) % parts;
  const uint64_t g = row / (limbs * parts);
  const DevPrime pr = primes[j];
  const uint64_t plane = (uint64_t)limbs << logn;  // one polynomial
  const uint64_t* c = ct + (g * count * parts + k) * plane + ((uint64_t)j << logn) + i;
  const uint64_t* p = pt + ((uint64_t)j << logn) + i;
  uint64_t hi = 0, lo = 0;
  for (uint32_t n = 0; n < count; n++) {
    mac128(hi, lo, c[(uint64_t)n * parts * plane], p[(uint64_t)n * plane]);
    if (n % 15 == 14) {
      lo = reduce128(hi, lo, pr);
      hi = 0;
    }
  }
  out[gid] = reduce128(hi, lo, pr);
}

// One level of the oblivious expansion for the `step` ciphertexts out[0..step):
// out[step + i] = (out[i] - sub[i]) * monomial when step + i < size, and
// out[i] += sub[i] (evaluation_key.rs:173-186).
__global__ void k_expand_step(const DevPrime* primes, uint64_t* out, const uint64_t* sub, const uint64_t* mono,
                              uint32_t step, uint32_t size, uint32_t limbs, uint32_t logn, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t row = row_of(gid, logn);  // (c, part, limb)
  const uint32_t j = row % limbs;
  const uint64_t c = row / (2 * limbs);
  const uint64_t ct_words = 2 * ((uint64_t)limbs << logn);
  const uint64_t off = gid - c * ct_words;  // within the ciphertext
  const DevPrime pr = primes[j];
  const uint64_t x = out[c * ct_words + off], y = sub[c * ct_words + off];
  if (step + c < size) {
    const uint64_t d = sub_mod(x, y, pr.p);
    out[(step + c) * ct_words + off] = mul_mod(d, mono[((uint64_t)j << logn) + i], pr);
  }
  out[c * ct_words + off] = add_mod(x, y, pr.p);
}

}  // namespace

void dot_product_scalar(const Params& par, size_t level, size_t parts, const uint64_t* cts, const uint64_t* pts,
                        uint64_t count, uint64_t groups, uint64_t* out, cudaStream_t st) {
  const Context& c = *par.ctx(level);
  const uint64_t total = groups * parts * c.L() << c.logn;
  if (total == 0) return;
  if (count == 0) throw Error(FHEG_ERR_INVALID_ARGUMENT, "At least one iterator is empty");
  k_dot_product<<<nblk(total, 256), 256, 0, st>>>(c.primes_dev(), cts, pts, out, (uint32_t)count, (uint32_t)parts,
                                                  (uint32_t)c.L(), c.logn, total);
  after_launch("k_dot_product");
}

void inner_sum(const Params& par, const Ksk* const* keys, const uint64_t* exponents, size_t nkeys,
               const uint64_t* ct, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st) {
  if (count == 0 || nkeys == 0) return;
  const size_t level = keys[0]->ciphertext_level;
  const Context& c = *par.ctx(level);
  const size_t words = count * 2 * c.L() * c.N();
  ws.reserve(words * 8 + 256);
  size_t off = 0;
  uint64_t* tmp = ws.take(words, &off);
  check_cuda(cudaMemcpyAsync(out, ct, words * 8, cudaMemcpyDeviceToDevice, st), "D2D");
  PolyRef o = plain_ref(out, c.L(), c.logn), t = plain_ref(tmp, c.L(), c.logn);
  for (size_t k = 0; k < nkeys; k++) {
    if (keys[k]->par != &par || keys[k]->ciphertext_level != level)
      throw Error(FHEG_ERR_KEY_MISMATCH, "all keys must share the parameters and the ciphertext level");
    galois_relinearize(*keys[k], exponents[k], out, tmp, count, keys[k]->ws, st);
    poly_op(c, 0, o, t, o, 2 * count, st);
  }
}

void expand(const Params& par, const Ksk* const* keys, const uint64_t* exponents, size_t nlevels, size_t size,
            const uint64_t* ct, uint64_t* out, Workspace& ws, cudaStream_t st) {
  if (size == 0) return;
  size_t level = 0;
  while (((size_t)1 << level) < size) level++;
  if (nlevels < level) throw Error(FHEG_ERR_INVALID_ARGUMENT, "not enough expansion keys for this size");
  if (level > 0 && keys[0]->par != &par) throw Error(FHEG_ERR_KEY_MISMATCH, "keys of other parameters");
  const size_t ct_level = level > 0 ? keys[0]->ciphertext_level : 0;
  const Context& c = *par.ctx(ct_level);
  const size_t L = c.L(), N = c.N();
  const size_t ct_words = 2 * L * N;
  check_cuda(cudaMemcpyAsync(out, ct, ct_words * 8, cudaMemcpyDeviceToDevice, st), "D2D");
  if (level == 0) return;
  const size_t half = (size_t)1 << (level - 1);
  ws.reserve((half * ct_words + level * L * N) * 8 + 512);
  size_t off = 0;
  uint64_t* sub = ws.take(half * ct_words, &off);
  uint64_t* mono = ws.take(level * L * N, &off);
  // evaluation_key.rs:355-363: monomial -x^(N - 2^l), Ntt.
  std::vector<uint64_t> h(level * L * N, 0);
  for (size_t l = 0; l < level; l++)
    for (size_t j = 0; j < L; j++) h[(l * L + j) * N + (N - ((size_t)1 << l))] = c.moduli[j] - 1;
  check_cuda(cudaMemcpyAsync(mono, h.data(), h.size() * 8, cudaMemcpyHostToDevice, st), "H2D");
  PolyRef mr = plain_ref(mono, L, c.logn);
  ntt_forward(c, mr, mr, level, false, st);
  for (size_t l = 0; l < level; l++) {
    const Ksk& k = *keys[l];
    if (k.ciphertext_level != ct_level) throw Error(FHEG_ERR_KEY_MISMATCH, "keys at different levels");
    const size_t step = (size_t)1 << l;
    galois_relinearize(k, exponents[l], out, sub, step, k.ws, st);
    const uint64_t total = step * ct_words;
    k_expand_step<<<nblk(total, 256), 256, 0, st>>>(c.primes_dev(), out, sub, mono + l * L * N, (uint32_t)step,
                                                    (uint32_t)size, (uint32_t)L, c.logn, total);
    after_launch("k_expand_step");
  }
}

}  // namespace fheg

using namespace fheg;

namespace {


std::vector<const Ksk*> key_list(const fheg_ksk* const* keys, size_t n) {
  std::vector<const Ksk*> out(n);
  for (size_t i = 0; i < n; i++) {
    abi_need(keys[i] != nullptr, "null key");
    out[i] = &keys[i]->k;
  }
  return out;
}

}  // namespace

FHEG_API int fheg_dot_product_scalar(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_cts,
                                     const uint64_t* d_pts, size_t count, size_t groups, uint64_t* d_out,
                                     void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && parts >= 1 && ((d_cts && d_pts && d_out) || !groups), "null input");
    dot_product_scalar(*par->p, level, parts, d_cts, d_pts, count, groups, d_out, static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_inner_sum(const fheg_params* par, const fheg_ksk* const* keys, const size_t* exponents,
                            size_t nkeys, const uint64_t* d_ct, uint64_t* d_out, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && keys && exponents && nkeys && ((d_ct && d_out) || !count), "null input");
    std::vector<uint64_t> ex(exponents, exponents + nkeys);
    const auto k = key_list(keys, nkeys);
    inner_sum(*par->p, k.data(), ex.data(), nkeys, d_ct, d_out, count, const_cast<fheg_params*>(par)->ws,
              static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_expand(const fheg_params* par, const fheg_ksk* const* keys, const size_t* exponents,
                         size_t nlevels, size_t size, const uint64_t* d_ct, uint64_t* d_out, void* stream) {
  return abi_call([&] {
    abi_need(par && d_ct && d_out && (nlevels == 0 || (keys && exponents)), "null input");
    std::vector<uint64_t> ex(exponents, exponents + nlevels);
    const auto k = key_list(keys, nlevels);
    expand(*par->p, k.data(), ex.data(), nlevels, size, d_ct, d_out, const_cast<fheg_params*>(par)->ws,
           static_cast<cudaStream_t>(stream));
  });
}
