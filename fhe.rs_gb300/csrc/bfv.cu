// BFV hot path (crate fhe): Multiplicator, key switching for
// relinearization and Galois rotations, ciphertext switch-down.
//
// Pipeline of Multiplicator::multiply (fhe/src/bfv/ops/mul.rs:158-227) for a
// batch of B ciphertext pairs at a level with L moduli and an extended basis
// of M moduli (each arrow is one kernel launch over the whole batch):
//   A  inverse NTT of the 4B input polynomials                (L limbs)
//   B  RNS basis extension Q -> Q u P per coefficient          (rns_scale)
//   C  forward NTT of the new limbs                            (M - L limbs)
//   D  tensor product fused into the inverse NTT               (3B x M limbs)
//   E  t/Q scale-and-round per coefficient                     (rns_scale)
//   F1 digit expansion: lazy forward NTT of every digit of c2 in every key
//      modulus (key_switching_key.rs:227-235, rq/mod.rs:518-540)
//   F2 forward NTT of c0, c1 fused with the key inner product and the final
//      additions (key_switching_key.rs:236-238, mul.rs:208-210)
// c2 is consumed in the power basis straight out of E: the reference's
// forward NTT of c2 followed by `into_power_basis` is the identity.

#include <algorithm>

#include "lib.hpp"
#include "ntt.cuh"

namespace fheg {

static unsigned nblocks(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

Params::Params(size_t n, const std::vector<uint64_t>& m, uint64_t t) : degree(n), moduli(m), plaintext(t) {
  if (m.empty()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "no moduli");
  levels.push_back(std::make_shared<Context>(m, n, nullptr));
  for (size_t l = 1; l < m.size(); l++) levels.push_back(levels[0]->prefix(m.size() - l));
}

const std::shared_ptr<Context>& Params::ctx(size_t level) const {
  if (level >= levels.size()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
  return levels[level];
}

// ---------------------------------------------------------------------------
// Functors for the fused NTTs.

// Four operands of a pair (lhs0, lhs1, rhs0, rhs1) as polynomials 4b .. 4b+3.
struct SrcPair {
  PolyRef lhs, rhs;  // [B][2][L][N]
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    const uint32_t b = j.poly >> 2, w = j.poly & 3;
    return w < 2 ? lhs.at(2 * b + w, j.limb)[i] : rhs.at(2 * b + w - 2, j.limb)[i];
  }
};

// Tensor product (mul.rs:181-185) at limb j of the extended basis: operand
// limbs below ncm come from the inputs, the others from the extension.
struct SrcTensor {
  PolyRef lhs, rhs;  // inputs [B][2][L][N], Ntt
  PolyRef ext;       // [B][4][M][N], Ntt (limbs >= ncm of each operand)
  uint32_t ncm_l, ncm_r;
  __device__ __forceinline__ uint64_t op(uint32_t b, uint32_t w, uint32_t limb, uint32_t i) const {
    const bool from_input = w < 2 ? limb < ncm_l : limb < ncm_r;
    if (from_input) return w < 2 ? lhs.at(2 * b + w, limb)[i] : rhs.at(2 * b + w - 2, limb)[i];
    return ext.at(4 * b + w, limb)[i];
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint32_t b = j.poly / 3, part = j.poly % 3;
    if (part == 0) return mul_mod(op(b, 0, j.limb, i), op(b, 2, j.limb, i), pr);
    if (part == 2) return mul_mod(op(b, 1, j.limb, i), op(b, 3, j.limb, i), pr);
    const uint64_t a0 = op(b, 0, j.limb, i), a1 = op(b, 1, j.limb, i);
    const uint64_t b0 = op(b, 2, j.limb, i), b1 = op(b, 3, j.limb, i);
    // a0*b1 + a1*b0 < 2^125: one reduction of the exact sum.
    const uint64_t lo1 = a0 * b1, hi1 = __umul64hi(a0, b1);
    const uint64_t lo2 = a1 * b0, hi2 = __umul64hi(a1, b0);
    const uint64_t lo = lo1 + lo2;
    const uint64_t hi = hi1 + hi2 + (lo < lo1);
    return reduce128(hi, lo, pr);
  }
};

// Digit i of c2 (power basis, mod q_i) lazily reduced modulo key limb j
// (rq/mod.rs:525-528).
struct SrcDigit {
  PolyRef digits;  // poly b * ndig + i -> row (b, i): stored as poly b, limb i
  uint32_t ndig;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint32_t b = j.poly / ndig, d = j.poly % ndig;
    return reduce64_lazy(digits.at(b, d)[i], pr);
  }
};

// Ntt input gathered through the substitution x -> x^e (rq/mod.rs:324-334).
__device__ __forceinline__ uint32_t brev_n(uint32_t x, uint32_t logn) { return __brev(x) >> (32 - logn); }
__device__ __forceinline__ uint32_t gather_index(uint32_t i, uint64_t e, uint32_t logn) {
  const uint64_t mask = (1ull << logn) - 1;
  return brev_n((uint32_t)((((e - 1) >> 1) + (uint64_t)brev_n(i, logn) * e) & mask), logn);
}

struct SrcSubst {
  PolyRef in;
  uint64_t e;
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return in.at(j.poly, j.limb)[gather_index(i, e, logn)];
  }
};

// Epilogue of F2: out = v + sum_d NTT(digit_d) * key_part[d] (mod q_j).
struct DstMac {
  PolyRef D;  // poly b * ndig + d, limb j (lazy NTT values)
  const uint64_t* k[2];
  const uint64_t* ks[2];
  PolyRef out;  // poly b * 2 + part
  uint32_t ndig, lk, logn;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime& pr, uint32_t i, uint64_t v) const {
    const uint32_t b = j.poly >> 1, part = j.poly & 1;
    uint64_t lo = v, hi = 0;
    const uint64_t* kp = k[part];
    const uint64_t* ksp = ks[part];
    for (uint32_t d = 0; d < ndig; d++) {
      const uint64_t off = (((uint64_t)d * lk + j.limb) << logn) + i;
      const uint64_t t = mul_shoup_lazy(D.at(b * ndig + d, j.limb)[i], __ldg(kp + off), __ldg(ksp + off), pr.p);
      lo += t;
      hi += lo < t;
    }
    out.at(j.poly, j.limb)[i] = reduce128(hi, lo, pr);
  }
};

// Element-wise inner product for relinearization / rotations:
// out_part[j] = add_part[j] + sum_d D[d][j] * key_part[d][j].
__global__ void k_key_mac(const DevPrime* primes, PolyRef D, const uint64_t* k0, const uint64_t* k0s,
                          const uint64_t* k1, const uint64_t* k1s, const uint64_t* add0, uint64_t add0_stride,
                          uint64_t add0_e, const uint64_t* add1, uint64_t add1_stride, uint64_t* out,
                          uint64_t out_stride, uint32_t ndig, uint32_t lk, uint32_t logn, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint64_t job = gid >> logn;
  const uint32_t j = job % lk;
  const uint32_t b = job / lk;
  const DevPrime pr = primes[j];
  uint64_t lo0 = 0, hi0 = 0, lo1 = 0, hi1 = 0;
  if (add0) lo0 = add0[b * add0_stride + ((uint64_t)j << logn) + (add0_e ? gather_index(i, add0_e, logn) : i)];
  if (add1) lo1 = add1[b * add1_stride + ((uint64_t)j << logn) + i];
  for (uint32_t d = 0; d < ndig; d++) {
    const uint64_t x = D.at(b * ndig + d, j)[i];
    const uint64_t off = (((uint64_t)d * lk + j) << logn) + i;
    const uint64_t t0 = mul_shoup_lazy(x, __ldg(k0 + off), __ldg(k0s + off), pr.p);
    const uint64_t t1 = mul_shoup_lazy(x, __ldg(k1 + off), __ldg(k1s + off), pr.p);
    lo0 += t0;
    hi0 += lo0 < t0;
    lo1 += t1;
    hi1 += lo1 < t1;
  }
  uint64_t* o = out + b * out_stride + ((uint64_t)j << logn) + i;
  o[0] = reduce128(hi0, lo0, pr);
  o[(uint64_t)lk << logn] = reduce128(hi1, lo1, pr);
}

// Shoup companions floor(v * 2^64 / p) of key values (zq/mod.rs:195-199).
__global__ void k_shoup(const DevPrime* primes, const uint64_t* v, uint64_t* out, uint32_t limbs, uint32_t logn,
                        uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t limb = (gid >> logn) % limbs;
  const DevPrime pr = primes[limb];
  const uint64_t x = v[gid];
  // Estimate with the Barrett constant, then correct (at most a few steps).
  uint64_t q = x * pr.bhi + __umul64hi(x, pr.blo);
  uint64_t plo = q * pr.p, phi = __umul64hi(q, pr.p);
  // r = x * 2^64 - q * p (128-bit, small and non-negative when q <= true q)
  uint64_t rlo = 0 - plo;
  uint64_t rhi = x - phi - (plo != 0);
  for (int it = 0; it < 4 && (rhi != 0 || rlo >= pr.p); it++) {
    const uint64_t nlo = rlo - pr.p;
    rhi -= (rlo < pr.p);
    rlo = nlo;
    q++;
  }
  out[gid] = q;
}

// ---------------------------------------------------------------------------
// Key switching (key_switching_key.rs:214-289) on digits in the power basis.

void key_switch(const Ksk& k, PolyRef digits, uint64_t batch, const uint64_t* add0, uint64_t add0_poly_stride,
                uint64_t add0_exponent, const uint64_t* add1, uint64_t add1_poly_stride, uint64_t* out,
                uint64_t out_poly_stride, uint64_t* D, cudaStream_t st) {
  const Context& kc = *k.ctx_ksk;
  const size_t Lk = kc.L(), nd = k.count;
  const uint32_t logn = kc.logn;
  PolyRef dref = plain_ref(D, Lk, logn);
  NttGeom g{kc.primes_dev(), (uint32_t)Lk, 0};
  // F1: every digit in every key modulus, lazy output (rq/mod.rs:518-540).
  ntt_forward_any<false>(logn, g, batch * nd, SrcDigit{digits, (uint32_t)nd}, DstPoly{dref}, st);
  const uint64_t total = batch * Lk << logn;
  k_key_mac<<<nblocks(total, 256), 256, 0, st>>>(kc.primes_dev(), dref, k.values(0), k.shoup(0), k.values(1),
                                                 k.shoup(1), add0, add0_poly_stride, add0_exponent, add1,
                                                 add1_poly_stride, out, out_poly_stride, (uint32_t)nd, (uint32_t)Lk,
                                                 logn, total);
  after_launch("k_key_mac");
}

void compute_shoup(const Context& c, const uint64_t* vals, uint64_t* out, uint64_t polys, cudaStream_t st) {
  const uint64_t total = polys * c.L() << c.logn;
  if (total == 0) return;
  k_shoup<<<nblocks(total, 256), 256, 0, st>>>(c.primes_dev(), vals, out, (uint32_t)c.L(), c.logn, total);
  after_launch("k_shoup");
}

static void require_same_level_key(const Ksk& k) {
  if (k.ctx_ksk->L() != k.ctx_ct->L())
    throw Error(FHEG_ERR_UNSUPPORTED, "key switching keys at a lower level than the ciphertext are not supported");
}

void relinearize(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st) {
  require_same_level_key(rk);
  const Context& c = *rk.ctx_ct;
  const size_t L = c.L(), N = c.N(), Lk = rk.ctx_ksk->L();
  if (count == 0) return;
  ws.buf.reserve((count * L * N + count * L * Lk * N + 64) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(count * L * N, &off);
  uint64_t* D = ws.take(count * L * Lk * N, &off);
  // relinearization_key.rs:81: c2 into the power basis.
  PolyRef src = sub_ref(const_cast<uint64_t*>(ct3), L, c.logn, 3, 2, 1);
  PolyRef dst = plain_ref(digits, L, c.logn);
  ntt_backward(c, src, dst, count, st);
  // relinearization_key.rs:82-95: key switch, then add to c0 and c1.
  key_switch(rk, dst, count, ct3, 3 * L * N, 0, ct3 + L * N, 3 * L * N, out, 2 * L * N, D, st);
}

// Relinearization with caller-provided scratch: `digits` holds count*L*N
// words and `D` count*L*Lk*N words. Same computation as relinearize().
void relinearize_scratch(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, uint64_t* digits,
                         uint64_t* D, cudaStream_t st) {
  require_same_level_key(rk);
  const Context& c = *rk.ctx_ct;
  const size_t L = c.L(), N = c.N();
  if (count == 0) return;
  PolyRef src = sub_ref(const_cast<uint64_t*>(ct3), L, c.logn, 3, 2, 1);
  PolyRef dst = plain_ref(digits, L, c.logn);
  ntt_backward(c, src, dst, count, st);
  key_switch(rk, dst, count, ct3, 3 * L * N, 0, ct3 + L * N, 3 * L * N, out, 2 * L * N, D, st);
}

void galois_relinearize(const Ksk& gk, uint64_t exponent, const uint64_t* ct, uint64_t* out, uint64_t count,
                        Workspace& ws, cudaStream_t st) {
  require_same_level_key(gk);
  const Context& c = *gk.ctx_ct;
  const size_t L = c.L(), N = c.N(), Lk = gk.ctx_ksk->L();
  const uint64_t e = exponent % (2 * N);
  if ((e & 1) == 0) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
  if (count == 0) return;
  ws.buf.reserve((count * L * N + count * L * Lk * N + 64) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(count * L * N, &off);
  uint64_t* D = ws.take(count * L * Lk * N, &off);
  // galois_key.rs:110: c2 = substitute(ct[1]) in the power basis; the
  // substitution is a gather fused into the inverse NTT.
  PolyRef src = sub_ref(const_cast<uint64_t*>(ct), L, c.logn, 2, 1, 1);
  PolyRef dst = plain_ref(digits, L, c.logn);
  NttGeom g{c.primes_dev(), (uint32_t)L, 0};
  ntt_inverse_any(c.logn, g, count, SrcSubst{src, e, c.logn}, DstPoly{dst}, st);
  // galois_key.rs:111-122: key switch, then out0 += substitute(ct[0]).
  key_switch(gk, dst, count, ct, 2 * L * N, e, nullptr, 0, out, 2 * L * N, D, st);
}

void ciphertext_switch_down(const Params& par, size_t level, size_t parts, uint64_t* ct, uint64_t* out,
                            uint64_t count, cudaStream_t st) {
  const Context& c = *par.ctx(level);
  if (level >= par.max_level()) throw Error(FHEG_ERR_NO_MORE_CONTEXT, "NoMoreContext");
  PolyRef in = plain_ref(ct, c.L(), c.logn);
  PolyRef o = plain_ref(out, c.L() - 1, c.logn);
  poly_switch_down_ntt(c, in, o, count * parts, st);
}

// ---------------------------------------------------------------------------
// Multiplicator

std::unique_ptr<Multiplicator> make_multiplicator(const Params& par, size_t level, const BigUint& lhs_n,
                                                  const BigUint& lhs_d, const BigUint& rhs_n, const BigUint& rhs_d,
                                                  const std::vector<uint64_t>& ext, const BigUint& post_n,
                                                  const BigUint& post_d) {
  auto m = std::unique_ptr<Multiplicator>(new Multiplicator());
  m->par = &par;
  m->level = level;
  m->base = par.ctx(level);
  // The extended basis reuses the roots of the moduli it shares with the base.
  std::vector<uint64_t> roots(ext.size(), 0);
  for (size_t i = 0; i < ext.size(); i++)
    for (size_t k = 0; k < m->base->L(); k++)
      if (ext[i] == m->base->moduli[k]) roots[i] = m->base->primes[k]->host.root;
  m->mul = std::make_shared<Context>(ext, par.degree, roots.data());
  m->ext_lhs.reset(new Scaler(m->base, m->mul, lhs_n, lhs_d));
  m->ext_rhs.reset(new Scaler(m->base, m->mul, rhs_n, rhs_d));
  m->down.reset(new Scaler(m->mul, m->base, post_n, post_d));
  if (m->down->number_common_moduli != 0)
    throw Error(FHEG_ERR_UNSUPPORTED, "a post-multiplication scaling factor of one is not supported");
  return m;
}

std::unique_ptr<Multiplicator> make_default_multiplicator(const Ksk& rk) {
  const Params& par = *rk.par;
  const Context& ctx = *par.ctx(rk.ciphertext_level);
  // mul.rs:104-117.
  size_t modulus_size = 0;
  for (uint64_t q : ctx.moduli) modulus_size += 64 - __builtin_clzll(q);
  const size_t n_moduli = (modulus_size + 60 + 61) / 62;
  std::vector<uint64_t> ext(ctx.moduli);
  uint64_t ub = (uint64_t)1 << 62;
  while (ext.size() != ctx.L() + n_moduli) {
    ub = generate_prime(62, 2 * (uint64_t)par.degree, ub);
    if (ub == 0) throw Error(FHEG_ERR_INTERNAL, "could not generate the extension basis");
    if (std::find(ext.begin(), ext.end(), ub) == ext.end()) ext.push_back(ub);
  }
  BigUint one(1), t(par.plaintext);
  auto m = make_multiplicator(par, rk.ciphertext_level, one, one, one, one, ext, t, ctx.rns->product);
  require_same_level_key(rk);
  m->rk = &rk;
  return m;
}

void Multiplicator::multiply(const uint64_t* lhs, const uint64_t* rhs, uint64_t* out, uint64_t count,
                             cudaStream_t st) {
  if (count == 0) return;
  const Context& bc = *base;
  const Context& mc = *mul;
  const size_t L = bc.L(), M = mc.L(), N = bc.N();
  const uint32_t logn = bc.logn;
  const size_t ncm_l = ext_lhs->number_common_moduli, ncm_r = ext_rhs->number_common_moduli;
  const size_t parts = out_parts();
  const size_t Lk = rk ? rk->ctx_ksk->L() : 0;
  // Workspace layout (words).
  const size_t w_pb = count * 4 * L * N, w_ext = count * 4 * M * N, w_prod = count * 3 * M * N,
               w_down = count * 3 * L * N, w_d = rk ? count * L * Lk * N : 0,
               w_tmp = mod_switch ? count * parts * L * N : 0;
  ws.buf.reserve((w_pb + w_ext + w_prod + w_down + w_d + w_tmp + 6 * 32) * 8);
  size_t off = 0;
  uint64_t* pb = ws.take(w_pb, &off);
  uint64_t* ext = ws.take(w_ext, &off);
  uint64_t* prod = ws.take(w_prod, &off);
  uint64_t* dn = ws.take(w_down, &off);
  uint64_t* D = ws.take(w_d, &off);
  uint64_t* tmp = ws.take(w_tmp, &off);
  uint64_t* dest = mod_switch ? tmp : out;

  PolyRef lref = plain_ref(const_cast<uint64_t*>(lhs), L, logn);
  PolyRef rref = plain_ref(const_cast<uint64_t*>(rhs), L, logn);
  PolyRef pbref = plain_ref(pb, L, logn);
  PolyRef extref = plain_ref(ext, M, logn);

  // A: inverse NTT of the four operands.
  {
    NttGeom g{bc.primes_dev(), (uint32_t)L, 0};
    ntt_inverse_any(logn, g, 4 * count, SrcPair{lref, rref}, DstPoly{pbref}, st);
  }
  // B + C: extension of each operand and forward NTT of the new limbs.
  const bool same_ext = ncm_l == ncm_r && ext_lhs->num == ext_rhs->num && ext_lhs->den == ext_rhs->den;
  auto extend = [&](const Scaler& s, uint32_t first, uint32_t take) {
    const size_t ncm = s.number_common_moduli;
    PolyRef in = sub_ref(pb, L, logn, 4, first, take);
    PolyRef o = sub_ref(ext, M, logn, 4, first, take);
    o.base += (uint64_t)ncm << logn;
    rns_scale(*s.rns, logn, in, o, (uint32_t)ncm, (uint32_t)(M - ncm), count * take, st);
    NttGeom g{mc.primes_dev() + ncm, (uint32_t)(M - ncm), 0};
    ntt_forward_any<true>(logn, g, count * take, SrcPoly{o}, DstPoly{o}, st);
  };
  if (same_ext) {
    extend(*ext_lhs, 0, 4);
  } else {
    extend(*ext_lhs, 0, 2);
    extend(*ext_rhs, 2, 2);
  }
  // D: tensor product fused into the inverse NTT over the extended basis.
  PolyRef prodref = plain_ref(prod, M, logn);
  {
    NttGeom g{mc.primes_dev(), (uint32_t)M, 0};
    ntt_inverse_any(logn, g, 3 * count, SrcTensor{lref, rref, extref, (uint32_t)ncm_l, (uint32_t)ncm_r},
                    DstPoly{prodref}, st);
  }
  // E: scale down by t/Q into the base context (power basis).
  PolyRef dnref = plain_ref(dn, L, logn);
  rns_scale(*down->rns, logn, prodref, dnref, 0, (uint32_t)L, 3 * count, st);
  NttGeom gb{bc.primes_dev(), (uint32_t)L, 0};
  if (rk) {
    // F1: digits of c2 in every key modulus.
    const Context& kc = *rk->ctx_ksk;
    PolyRef dref = plain_ref(D, Lk, logn);
    PolyRef c2 = sub_ref(dn, L, logn, 3, 2, 1);
    NttGeom gk{kc.primes_dev(), (uint32_t)Lk, 0};
    ntt_forward_any<false>(logn, gk, count * L, SrcDigit{c2, (uint32_t)L}, DstPoly{dref}, st);
    // F2: forward NTT of c0, c1 with the key inner product in the epilogue.
    PolyRef c01 = sub_ref(dn, L, logn, 3, 0, 2);
    DstMac mac;
    mac.D = dref;
    mac.k[0] = rk->values(0);
    mac.k[1] = rk->values(1);
    mac.ks[0] = rk->shoup(0);
    mac.ks[1] = rk->shoup(1);
    mac.out = plain_ref(dest, L, logn);
    mac.ndig = (uint32_t)L;
    mac.lk = (uint32_t)Lk;
    mac.logn = logn;
    if (logn <= kMaxSmemLogN) {
      ntt_fwd_single<true>(logn, gb, 2 * count, SrcPoly{c01}, mac, st);
    } else {
      // Two-pass sizes: forward into the output, then apply the inner product.
      PolyRef o = plain_ref(dest, L, logn);
      ntt_forward_any<true>(logn, gb, 2 * count, SrcPoly{c01}, DstPoly{o}, st);
      const uint64_t total = count * L << logn;
      k_key_mac<<<nblocks(total, 256), 256, 0, st>>>(bc.primes_dev(), dref, rk->values(0), rk->shoup(0),
                                                     rk->values(1), rk->shoup(1), dest, 2 * L * N, 0, dest + L * N,
                                                     2 * L * N, dest, 2 * L * N, (uint32_t)L, (uint32_t)Lk, logn,
                                                     total);
      after_launch("k_key_mac");
    }
  } else {
    PolyRef o = plain_ref(dest, L, logn);
    ntt_forward_any<true>(logn, gb, 3 * count, SrcPoly{dnref}, DstPoly{o}, st);
  }
  if (mod_switch) {
    PolyRef in = plain_ref(tmp, L, logn);
    PolyRef o = plain_ref(out, L - 1, logn);
    poly_switch_down_ntt(bc, in, o, count * parts, st);
  }
}

}  // namespace fheg
