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
//   F  one launch of forward NTTs: every digit of c2 in every key modulus
//      (key_switching_key.rs:227-235, rq/mod.rs:518-540) and c0, c1
//   G  key inner product and the final additions, exact 128-bit sums
//      reduced once (key_switching_key.rs:236-238, mul.rs:208-210)
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
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    const uint32_t b = j.poly >> 2, w = j.poly & 3;
    prefetch_l2(w < 2 ? lhs.at(2 * b + w, j.limb) + i : rhs.at(2 * b + w - 2, j.limb) + i);
  }
};

// Tensor product (mul.rs:181-185) at limb j of the extended basis: operand
// limbs below ncm come from the inputs, the others from the extension. The
// products are Montgomery reductions (value * 2^-64 mod q_j, in [0, 2q_j));
// the inverse NTT that consumes them scales by N^-1 * 2^64 instead of N^-1,
// so its output is the canonical INTT of the exact products.
struct SrcTensor {
  static constexpr bool kMontgomery = true;
  static constexpr bool kStaged = true;
  PolyRef lhs, rhs;  // inputs [B][2][L][N], Ntt
  PolyRef ext;       // [B][4][M][N], Ntt (limbs >= ncm of each operand)
  uint32_t ncm_l, ncm_r;
  __device__ __forceinline__ const uint64_t* row(uint32_t b, uint32_t w, uint32_t limb) const {
    const bool from_input = w < 2 ? limb < ncm_l : limb < ncm_r;
    if (from_input) return w < 2 ? lhs.at(2 * b + w, limb) : rhs.at(2 * b + w - 2, limb);
    return ext.at(4 * b + w, limb);
  }
  __device__ __forceinline__ uint64_t op(uint32_t b, uint32_t w, uint32_t limb, uint32_t i) const {
    return row(b, w, limb)[i];
  }
  // Staged load for the inverse NTT (k_ntt_inv): the operand rows stream
  // into shared memory with asynchronous copies, half a block at a time (the
  // two operands of a product fill the buffer), so every load of the phase is
  // in flight at once instead of what the registers can hold; the products of
  // the cross term are Montgomery-reduced separately and added (both carry
  // the factor 2^-64).
  template <int LOGN, int T, int E>
  __device__ __forceinline__ void stage(const NttJob& j, const DevPrime& pr, uint32_t base, uint64_t* sm,
                                        uint32_t tid, uint64_t* x) const {
    constexpr uint32_t HALF = 1u << (LOGN - 1);
    const uint32_t b = j.poly / 3, part = j.poly % 3;
    const int npairs = part == 1 ? 2 : 1;
#pragma unroll
    for (int h = 0; h < 2; h++) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        if (q < npairs) {
          // part 0: l0 r0; part 2: l1 r1; part 1: l0 r1 + l1 r0.
          const uint32_t wa = part == 0 ? 0 : (part == 2 ? 1 : (uint32_t)q);
          const uint32_t wb = part == 0 ? 2 : (part == 2 ? 3 : (q == 0 ? 3u : 2u));
          const uint64_t* ra = row(b, wa, j.limb) + base + h * HALF;
          const uint64_t* rb = row(b, wb, j.limb) + base + h * HALF;
          for (uint32_t c = tid; c < HALF / 2; c += T) {
            cp_async16(sm + 2 * c, ra + 2 * c);
            cp_async16(sm + HALF + 2 * c, rb + 2 * c);
          }
          cp_async_wait_all();
          __syncthreads();
#pragma unroll
          for (int e = 0; e < E / 2; e++) {
            const uint32_t idx = tid + e * T;
            const uint64_t u = sm[idx], v = sm[HALF + idx];
            const uint64_t m = mont_reduce(__umul64hi(u, v), u * v, pr);
            x[h * (E / 2) + e] = q == 0 ? m : csub(x[h * (E / 2) + e] + m, pr.p2);
          }
          __syncthreads();
        }
      }
    }
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    const uint32_t b = j.poly / 3, part = j.poly % 3;
    if (part != 2) {
      prefetch_l2(row(b, 0, j.limb) + i);
      prefetch_l2(row(b, 2, j.limb) + i);
    }
    if (part != 0) {
      prefetch_l2(row(b, 1, j.limb) + i);
      prefetch_l2(row(b, 3, j.limb) + i);
    }
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint32_t b = j.poly / 3, part = j.poly % 3;
    if (part != 1) {
      const uint64_t x = op(b, part >> 1, j.limb, i), y = op(b, 2 + (part >> 1), j.limb, i);
      return mont_reduce(__umul64hi(x, y), x * y, pr);
    }
    const uint64_t a0 = op(b, 0, j.limb, i), a1 = op(b, 1, j.limb, i);
    const uint64_t b0 = op(b, 2, j.limb, i), b1 = op(b, 3, j.limb, i);
    // a0*b1 + a1*b0 < 2 q_j^2 < q_j * 2^64: one reduction of the exact sum.
    uint64_t hi = 0, lo = 0;
    mac128(hi, lo, a0, b1);
    mac128(hi, lo, a1, b0);
    return mont_reduce(hi, lo, pr);
  }
};

// Montgomery products already in memory (the split form of stage D).
struct SrcPolyMont {
  static constexpr bool kMontgomery = true;
  PolyRef r;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return r.at(j.poly, j.limb)[i];
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const { prefetch_l2(r.at(j.poly, j.limb) + i); }
};

// The tensor products of SrcTensor as an element-wise kernel: one thread per
// (product polynomial, limb, coefficient).
__global__ void k_tensor(const DevPrime* primes, SrcTensor t, PolyRef out, uint32_t limbs, uint32_t logn,
                         uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  NttJob j;
  j.limb = (uint32_t)(job % limbs);
  j.poly = (uint32_t)(job / limbs);
  j.beta = 0;
  j.aux = 0;
  const DevPrime pr = primes[j.limb];
  out.at(j.poly, j.limb)[i] = t(j, pr, i);
}

// Digit i of c2 (power basis, mod q_i) lazily reduced modulo key limb j
// (rq/mod.rs:525-528).
// With `raw` set every digit modulus is below 4 q_j, so the digit already
// lies in the forward NTT's input range [0, 4 q_j) and needs no reduction
// (the transform is the same modulo q_j).
struct SrcDigit {
  PolyRef digits;  // poly b * ndig + i -> row (b, i): stored as poly b, limb i
  uint32_t ndig;
  uint32_t raw;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint32_t b = j.poly / ndig, d = j.poly % ndig;
    const uint64_t x = digits.at(b, d)[i];
    return raw ? x : reduce64_lazy(x, pr);
  }

  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    prefetch_l2(digits.at(j.poly / ndig, j.poly % ndig) + i);
  }
};

// Ntt input gathered through the substitution x -> x^e (rq/mod.rs:324-334).
__device__ __forceinline__ uint32_t brev_n(uint32_t x, uint32_t logn) { return __brev(x) >> (32 - logn); }
__device__ __forceinline__ uint32_t gather_index(uint32_t i, uint64_t e, uint32_t logn) {
  const uint64_t mask = (1ull << logn) - 1;
  return brev_n((uint32_t)((((e - 1) >> 1) + (uint64_t)brev_n(i, logn) * e) & mask), logn);
}

// Staged gather: when the block is the whole row (single-pass transforms),
// the row streams into shared memory with asynchronous copies and the
// permutation reads it there instead of scattering 8-byte reads over DRAM;
// otherwise the elements are gathered from global memory.
template <int LOGN, int T, int E>
__device__ __forceinline__ void stage_gather(const uint64_t* row, uint64_t e, uint32_t logn, uint32_t base,
                                             uint64_t* sm, uint32_t tid, uint64_t* x) {
  if (logn != (uint32_t)LOGN || (reinterpret_cast<uintptr_t>(row) & 15) != 0) {
#pragma unroll
    for (int k = 0; k < E; k++) x[k] = row[gather_index(base + tid + k * T, e, logn)];
    return;
  }
  for (uint32_t c = tid; c < (1u << LOGN) / 2; c += T) cp_async16(sm + 2 * c, row + 2 * c);
  cp_async_wait_all();
  __syncthreads();
#pragma unroll
  for (int k = 0; k < E; k++) x[k] = sm[gather_index(tid + k * T, e, logn)];
  __syncthreads();
}

struct SrcSubst {
  static constexpr bool kStaged = true;
  PolyRef in;
  uint64_t e;
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return in.at(j.poly, j.limb)[gather_index(i, e, logn)];
  }
  template <int LOGN, int T, int E>
  __device__ __forceinline__ void stage(const NttJob& j, const DevPrime&, uint32_t base, uint64_t* sm, uint32_t tid,
                                        uint64_t* x) const {
    stage_gather<LOGN, T, E>(in.at(j.poly, j.limb), e, logn, base, sm, tid, x);
  }
  // The gather reads the whole row: hint its lines in order.
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const { prefetch_l2(in.at(j.poly, j.limb) + i); }
};

// F stage of the multiplication: polynomials [0, B*L) are the digits of c2
// (digit d of ciphertext b is polynomial b*L + d, lazily reduced into key
// limb j), polynomials [B*L, B*L + 2B) are c0 and c1 of each product.
struct SrcKsF {
  PolyRef digits;  // c2 rows: poly b, limb d
  PolyRef c01;     // c0 / c1: poly 2b + part
  uint32_t ndig, ndig_polys;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    if (j.poly < ndig_polys) return reduce64_lazy(digits.at(j.poly / ndig, j.poly % ndig)[i], pr);
    return c01.at(j.poly - ndig_polys, j.limb)[i];
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    if (j.poly < ndig_polys) prefetch_l2(digits.at(j.poly / ndig, j.poly % ndig) + i);
    else prefetch_l2(c01.at(j.poly - ndig_polys, j.limb) + i);
  }
};

struct DstKsF {
  PolyRef D;    // poly b*L + d
  PolyRef out;  // poly 2b + part
  uint32_t ndig_polys;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    if (j.poly < ndig_polys) D.at(j.poly, j.limb)[i] = v;
    else out.at(j.poly - ndig_polys, j.limb)[i] = v;
  }
};

// Key inner product for relinearization, rotations and the multiplication:
// out_part[j] = add_part[j] + sum_d D[d][j] * key_part[d][j] (mod q_j), with
// D and the keys canonical, so each product is below 2^124 and up to 15
// products are summed exactly before a Barrett reduction. A thread handles
// one residue of limb j for KB ciphertexts of the batch (each key residue is
// then read once per KB ciphertexts).
// D is a plain array [batch * ndig][lk][N] (digit d of ciphertext b at row
// b * ndig + d, dstride words apart), addressed directly: a PolyRef lookup
// per digit would cost a division per residue.
template <int KB>
__global__ void k_key_mac(const DevPrime* primes, const uint64_t* D, uint64_t dstride, const uint64_t* k0,
                          const uint64_t* k1,
                          const uint64_t* add0, uint64_t add0_stride, uint64_t add0_e, const uint64_t* add1,
                          uint64_t add1_stride, uint64_t* out, uint64_t out_stride, uint32_t ndig, uint32_t lk,
                          uint32_t logn, uint64_t batch, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t j = job % lk;
  const uint64_t b0 = (uint64_t)(job / lk) * KB;
  const DevPrime pr = primes[j];
  uint64_t lo0[KB], hi0[KB], lo1[KB], hi1[KB];
  const uint32_t gi = add0_e ? gather_index(i, add0_e, logn) : i;
#pragma unroll
  for (int u = 0; u < KB; u++) {
    const uint64_t b = b0 + u;
    lo0[u] = hi0[u] = lo1[u] = hi1[u] = 0;
    if (b < batch) {
      if (add0) lo0[u] = add0[b * add0_stride + ((uint64_t)j << logn) + gi];
      if (add1) lo1[u] = add1[b * add1_stride + ((uint64_t)j << logn) + i];
    }
  }
  const uint64_t kstride = (uint64_t)lk << logn;
  const uint64_t* kp0 = k0 + ((uint64_t)j << logn) + i;
  const uint64_t* kp1 = k1 + ((uint64_t)j << logn) + i;
  for (uint32_t d = 0; d < ndig; d++) {
    const uint64_t w0 = __ldg(kp0 + d * kstride), w1 = __ldg(kp1 + d * kstride);
#pragma unroll
    for (int u = 0; u < KB; u++) {
      const uint64_t b = b0 + u;
      if (b < batch) {
        const uint64_t x = D[(b * ndig + d) * dstride + ((uint64_t)j << logn) + i];
        mac128(hi0[u], lo0[u], x, w0);
        mac128(hi1[u], lo1[u], x, w1);
      }
    }
    if (d % 15 == 14) {
#pragma unroll
      for (int u = 0; u < KB; u++) {
        lo0[u] = reduce128(hi0[u], lo0[u], pr);
        hi0[u] = 0;
        lo1[u] = reduce128(hi1[u], lo1[u], pr);
        hi1[u] = 0;
      }
    }
  }
#pragma unroll
  for (int u = 0; u < KB; u++) {
    const uint64_t b = b0 + u;
    if (b < batch) {
      uint64_t* o = out + b * out_stride + ((uint64_t)j << logn) + i;
      o[0] = reduce128(hi0[u], lo0[u], pr);
      o[kstride] = reduce128(hi1[u], lo1[u], pr);
    }
  }
}

// Launches k_key_mac over `batch` ciphertexts, one per thread: sharing the
// key loads among 4 ciphertexts per thread measured 60% slower on GB300 at 64
// pairs (fewer threads left too little parallelism to cover the loads of D).
void launch_key_mac(const DevPrime* primes, PolyRef D, const uint64_t* k0, const uint64_t* k1, const uint64_t* add0,
                    uint64_t add0_stride, uint64_t add0_e, const uint64_t* add1, uint64_t add1_stride, uint64_t* out,
                    uint64_t out_stride, uint32_t ndig, uint32_t lk, uint32_t logn, uint64_t batch, cudaStream_t st) {
  if (batch == 0) return;
  if (D.grp != 1) throw Error(FHEG_ERR_INTERNAL, "key inner product: digits must be a plain array");
  const uint64_t total = batch * lk << logn;
  k_key_mac<1><<<nblocks(total, 256), 256, 0, st>>>(primes, D.base, D.grp_stride, k0, k1, add0, add0_stride, add0_e,
                                                    add1, add1_stride, out, out_stride, ndig, lk, logn, batch, total);
  after_launch("k_key_mac");
}

// Whether digits of `digit_moduli` can enter NTTs modulo `key_moduli`
// unreduced: every digit is below four times every key modulus (moduli are
// below 2^62, so 4 q does not overflow).
static uint32_t digits_fit(const std::vector<uint64_t>& digit_moduli, const std::vector<uint64_t>& key_moduli) {
  uint64_t dmax = 0, kmin = ~0ull;
  for (uint64_t q : digit_moduli) dmax = std::max(dmax, q);
  for (uint64_t q : key_moduli) kmin = std::min(kmin, q);
  return dmax <= 4 * kmin ? 1u : 0u;
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
  // Every digit in every key modulus (rq/mod.rs:518-540), reduced output.
  ntt_forward_any<true>(logn, g, batch * nd,
                        SrcDigit{digits, (uint32_t)nd, digits_fit(k.ctx_ct->moduli, kc.moduli)}, DstPoly{dref}, st);
  launch_key_mac(kc.primes_dev(), dref, k.values(0), k.values(1), add0, add0_poly_stride, add0_exponent, add1,
                 add1_poly_stride, out, out_poly_stride, (uint32_t)nd, (uint32_t)Lk, logn, batch, st);
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
  ws.reserve((count * L * N + count * L * Lk * N + 64) * 8);
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
  ws.reserve((count * L * N + count * L * Lk * N + 64) * 8);
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

// Mul<&RGSWCiphertext> for &Ciphertext (rgsw_ciphertext.rs:123-153): the
// reference key-switches ct0 with ksk0 and ct1 with ksk1 and adds the two
// results. `rgsw` holds both keys as one key of 2L digits per part (ksk0's
// digits, then ksk1's), so the two key switches and their sum are one
// digit NTT launch and one key inner product over the 2L rows of
// (ct0, ct1) in the power basis.
void external_product(const Ksk& rgsw, const uint64_t* ct, uint64_t* out, uint64_t count, Workspace& ws,
                      cudaStream_t st) {
  const Context& c = *rgsw.ctx_ct;
  const size_t L = c.L(), N = c.N(), Lk = rgsw.ctx_ksk->L();
  if (rgsw.count != 2 * L || Lk != L) throw Error(FHEG_ERR_INTERNAL, "malformed RGSW key");
  if (count == 0) return;
  ws.reserve((count * 2 * L * N + count * 2 * L * Lk * N + 64) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(count * 2 * L * N, &off);
  uint64_t* D = ws.take(count * 2 * L * Lk * N, &off);
  // rgsw_ciphertext.rs:137-138: both parts into the power basis.
  ntt_backward(c, plain_ref(const_cast<uint64_t*>(ct), L, c.logn), plain_ref(digits, L, c.logn), 2 * count, st);
  // rgsw_ciphertext.rs:140-152: digit i < L is row i of ct0, digit L + i row i of ct1.
  key_switch(rgsw, plain_ref(digits, 2 * L, c.logn), count, nullptr, 0, 0, nullptr, 0, out, 2 * L * N, D, st);
}

// ---------------------------------------------------------------------------
// Ragged rotation batch: GaloisKey::relinearize_into (galois_key.rs:90-124)
// for ciphertexts at different levels, each with its own key and exponent,
// in one launch per stage. Levels are prefixes of one moduli chain, so limb
// j of every ciphertext uses modulus j.

struct RotDesc {
  const uint64_t* ct;  // [2][L][N] Ntt
  uint64_t* out;       // [2][L][N] Ntt
  uint64_t* digits;    // [L][N] scratch: substituted c1 in the power basis
  uint64_t* D;         // [L digits][L limbs][N] scratch: digit NTTs
  const uint64_t* k0;  // [L][L][N] key values, part 0
  const uint64_t* k1;  // part 1
  uint64_t e;          // substitution exponent mod 2N
  uint32_t L, pad;
};

// R1: substituted c1, gathered into the inverse NTT (jobs: poly = b, limb = i).
struct SrcRotSubst {
  static constexpr bool kStaged = true;
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    const RotDesc& r = d[j.poly];
    return r.ct[((uint64_t)(r.L + j.limb) << logn) + gather_index(i, r.e, logn)];
  }
  template <int LOGN, int T, int E>
  __device__ __forceinline__ void stage(const NttJob& j, const DevPrime&, uint32_t base, uint64_t* sm, uint32_t tid,
                                        uint64_t* x) const {
    const RotDesc& r = d[j.poly];
    stage_gather<LOGN, T, E>(r.ct + ((uint64_t)(r.L + j.limb) << logn), r.e, logn, base, sm, tid, x);
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    const RotDesc& r = d[j.poly];
    prefetch_l2(r.ct + ((uint64_t)(r.L + j.limb) << logn) + i);
  }
};

struct DstRotDigits {
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    d[j.poly].digits[((uint64_t)j.limb << logn) + i] = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const {
    return d[j.poly].digits[((uint64_t)j.limb << logn) + i];
  }
};

// F: digit `aux` of ciphertext `poly` in key limb `limb`.
struct SrcRotDigit {
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    return reduce64_lazy(d[j.poly].digits[((uint64_t)j.aux << logn) + i], pr);
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    prefetch_l2(d[j.poly].digits + ((uint64_t)j.aux << logn) + i);
  }
};

struct DstRotD {
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ uint64_t* at(const NttJob& j, uint32_t i) const {
    const RotDesc& r = d[j.poly];
    return r.D + ((uint64_t)(j.aux * r.L + j.limb) << logn) + i;
  }
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    *at(j, i) = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const { return *at(j, i); }
};

// G: out0 = substitute(ct0) + sum_d D[d] * k0[d], out1 = sum_d D[d] * k1[d]
// for row (poly, limb) = rows[blockIdx.y]; exact sums reduced once.
__global__ void k_rot_mac(const DevPrime* primes, const RotDesc* d, const uint2* rows, uint32_t logn) {
  const uint2 row = rows[blockIdx.y];
  const RotDesc& r = d[row.x];
  const uint32_t j = row.y;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << logn)) return;
  const DevPrime pr = primes[j];
  const uint64_t plane = (uint64_t)r.L << logn;
  uint64_t lo0 = r.ct[((uint64_t)j << logn) + gather_index(i, r.e, logn)], hi0 = 0, lo1 = 0, hi1 = 0;
  for (uint32_t dd = 0; dd < r.L; dd++) {
    const uint64_t off = ((uint64_t)(dd * r.L + j) << logn) + i;
    const uint64_t x = r.D[off];
    mac128(hi0, lo0, x, __ldg(r.k0 + off));
    mac128(hi1, lo1, x, __ldg(r.k1 + off));
    if (dd % 15 == 14) {
      lo0 = reduce128(hi0, lo0, pr);
      hi0 = 0;
      lo1 = reduce128(hi1, lo1, pr);
      hi1 = 0;
    }
  }
  r.out[((uint64_t)j << logn) + i] = reduce128(hi0, lo0, pr);
  r.out[plane + ((uint64_t)j << logn) + i] = reduce128(hi1, lo1, pr);
}

size_t galois_batch_scratch_bytes(const RotRequest* req, size_t count) {
  size_t words = 0, n_r1 = 0, n_f = 0;
  for (size_t b = 0; b < count; b++) {
    const size_t L = req[b].key->ctx_ct->L(), N = req[b].key->ctx_ct->N();
    words += L * N + L * L * N;
    n_r1 += L;
    n_f += L * L;
  }
  const size_t table_words = (count * sizeof(RotDesc) + (n_r1 + n_f) * sizeof(uint4) + n_r1 * sizeof(uint2)) / 8 + 8;
  return (words + table_words + 128 + 3 * 32) * 8;
}

void galois_relinearize_batch(const Params& par, const RotRequest* req, size_t count, Workspace& ws,
                              cudaStream_t st) {
  if (count == 0) return;
  const Context& top = *par.ctx(0);
  const size_t N = top.N();
  const uint32_t logn = top.logn;
  // Scratch and tables.
  size_t digit_words = 0, d_words = 0, n_r1 = 0, n_f = 0;
  for (size_t b = 0; b < count; b++) {
    const Ksk& k = *req[b].key;
    if (k.par != &par) throw Error(FHEG_ERR_KEY_MISMATCH, "all keys of a batch must share the parameters");
    require_same_level_key(k);
    if ((req[b].exponent % (2 * N)) % 2 == 0)
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
    const size_t L = k.ctx_ct->L();
    digit_words += L * N;
    d_words += L * L * N;
    n_r1 += L;
    n_f += L * L;
  }
  std::vector<RotDesc> desc(count);
  std::vector<uint4> jobs;
  jobs.reserve(n_r1 + n_f);
  std::vector<uint2> rows;
  rows.reserve(n_r1);
  const size_t table_words = (count * sizeof(RotDesc) + (n_r1 + n_f) * sizeof(uint4) + n_r1 * sizeof(uint2)) / 8 + 8;
  ws.reserve((digit_words + d_words + table_words + 128) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(digit_words, &off);
  uint64_t* D = ws.take(d_words, &off);
  uint64_t* tables = ws.take(table_words, &off);
  size_t dpos = 0, Dpos = 0;
  for (size_t b = 0; b < count; b++) {
    const Ksk& k = *req[b].key;
    const uint32_t L = (uint32_t)k.ctx_ct->L();
    RotDesc& r = desc[b];
    r.ct = req[b].ct;
    r.out = req[b].out;
    r.digits = digits + dpos;
    r.D = D + Dpos;
    r.k0 = k.values(0);
    r.k1 = k.values(1);
    r.e = req[b].exponent % (2 * N);
    r.L = L;
    r.pad = 0;
    dpos += (size_t)L * N;
    Dpos += (size_t)L * L * N;
    for (uint32_t i = 0; i < L; i++) jobs.push_back(make_uint4((uint32_t)b, i, 0, 0));
  }
  for (size_t b = 0; b < count; b++)
    for (uint32_t dd = 0; dd < desc[b].L; dd++)
      for (uint32_t j = 0; j < desc[b].L; j++) jobs.push_back(make_uint4((uint32_t)b, j, dd, 0));
  for (size_t b = 0; b < count; b++)
    for (uint32_t j = 0; j < desc[b].L; j++) rows.push_back(make_uint2((uint32_t)b, j));
  // Upload the tables (pageable source: the copy completes before return).
  uint8_t* tb = reinterpret_cast<uint8_t*>(tables);
  RotDesc* d_desc = reinterpret_cast<RotDesc*>(tb);
  uint4* d_jobs = reinterpret_cast<uint4*>(tb + count * sizeof(RotDesc));
  uint2* d_rows = reinterpret_cast<uint2*>(tb + count * sizeof(RotDesc) + jobs.size() * sizeof(uint4));
  check_cuda(cudaMemcpyAsync(d_desc, desc.data(), count * sizeof(RotDesc), cudaMemcpyHostToDevice, st), "H2D");
  check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(uint4), cudaMemcpyHostToDevice, st), "H2D");
  check_cuda(cudaMemcpyAsync(d_rows, rows.data(), rows.size() * sizeof(uint2), cudaMemcpyHostToDevice, st), "H2D");
  // R1: substituted c1 into the power basis.
  NttGeom g1{top.primes_dev(), 1, 0, d_jobs};
  ntt_inverse_any(logn, g1, n_r1, SrcRotSubst{d_desc, logn}, DstRotDigits{d_desc, logn}, st);
  // F: every digit in every key limb.
  NttGeom g2{top.primes_dev(), 1, 0, d_jobs + n_r1};
  ntt_forward_any<true>(logn, g2, n_f, SrcRotDigit{d_desc, logn}, DstRotD{d_desc, logn}, st);
  // G: inner products and the substituted c0.
  dim3 grid((unsigned)((N + 255) / 256), (unsigned)rows.size());
  k_rot_mac<<<grid, 256, 0, st>>>(top.primes_dev(), d_desc, d_rows, logn);
  after_launch("k_rot_mac");
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

size_t Multiplicator::scratch_bytes(uint64_t count) const {
  const size_t L = base->L(), M = mul->L(), N = base->N();
  const size_t Lk = rk ? rk->ctx_ksk->L() : 0;
  const size_t words = count * 4 * L * N + count * 4 * M * N + count * 3 * M * N + count * 3 * L * N +
                       (rk ? count * L * Lk * N : 0) + (mod_switch ? count * out_parts() * L * N : 0) + 6 * 32;
  return words * 8;
}

void Multiplicator::multiply(const uint64_t* lhs, const uint64_t* rhs, uint64_t* out, uint64_t count,
                             cudaStream_t st, Workspace* scratch, cudaEvent_t* marks) {
  if (count == 0) return;
  auto mark = [&](int k) {
    if (marks) check_cuda(cudaEventRecord(marks[k], st), "cudaEventRecord");
  };
  Workspace& ws = scratch ? *scratch : this->ws;
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
  ws.reserve(scratch_bytes(count));
  size_t off = 0;
  uint64_t* pb = ws.take(w_pb, &off);
  uint64_t* ext = ws.take(w_ext, &off);
  uint64_t* prod = ws.take(w_prod, &off);
  uint64_t* dn = ws.take(w_down, &off);
  uint64_t* D = ws.take(w_d, &off);
  uint64_t* tmp = ws.take(w_tmp, &off);
  uint64_t* dest = mod_switch ? tmp : out;

  // Stage plans: the small-batch plan when it applies.
  uint32_t plan_a = this->plan_a, plan_c = this->plan_c, plan_d = this->plan_d, plan_f = this->plan_f;
  bool f_split = this->f_split, tensor_split = this->tensor_split;
  if (count <= small_count && ntt_plan_valid(logn, small_plan[0]) && ntt_plan_valid(logn, small_plan[1]) &&
      ntt_plan_valid(logn, small_plan[2]) && ntt_plan_valid(logn, small_plan[3])) {
    plan_a = small_plan[0];
    plan_c = small_plan[1];
    plan_d = small_plan[2];
    plan_f = small_plan[3];
    f_split = small_plan[4] != 0;
    tensor_split = small_plan[5] != 0;
  }

  PolyRef lref = plain_ref(const_cast<uint64_t*>(lhs), L, logn);
  PolyRef rref = plain_ref(const_cast<uint64_t*>(rhs), L, logn);
  PolyRef pbref = plain_ref(pb, L, logn);
  PolyRef extref = plain_ref(ext, M, logn);

  // Strided last stages of a two-pass inverse NTT that the RNS scaler after
  // it can apply while loading (its only consumer): 0 when the plan is single
  // pass or the scaler cannot.
  auto top_stages = [&](uint32_t plan, const Scaler& s1c, const Scaler* s2c, uint32_t out_len) -> uint32_t {
    const uint32_t bl = plan ? plan : ntt_block_logn(logn);
    if (bl >= logn || logn < 13) return 0;
    const uint32_t s1 = logn - bl;
    if (!rns_scale_takes_top(*s1c.rns, logn, out_len, s1)) return 0;
    if (s2c && !rns_scale_takes_top(*s2c->rns, logn, out_len, s1)) return 0;
    return s1;
  };

  // A: inverse NTT of the four operands (without its strided last stages
  // when B applies them).
  mark(0);
  const uint32_t top_a = top_stages(plan_a, *ext_lhs, ext_rhs.get(), (uint32_t)(M - std::min(ncm_l, ncm_r)));
  {
    NttGeom g{bc.primes_dev(), (uint32_t)L, 0};
    if (top_a) ntt_inverse_blocks(logn, g, 4 * count, SrcPair{lref, rref}, DstPoly{pbref}, st, plan_a);
    else ntt_inverse_any(logn, g, 4 * count, SrcPair{lref, rref}, DstPoly{pbref}, st, plan_a);
  }
  const InverseTop top_a_args{top_a, 0u, bc.primes_dev()};
  mark(1);
  // B + C: extension of each operand and forward NTT of the new limbs.
  const bool same_ext = ncm_l == ncm_r && ext_lhs->num == ext_rhs->num && ext_lhs->den == ext_rhs->den;
  // C's strided first stages run in B's epilogue when both transforms have
  // the same number of them (B then writes C's block-pass input).
  const uint32_t bl_c = plan_c ? plan_c : ntt_block_logn(logn);
  const bool fuse_c = top_a && bl_c < logn && logn - bl_c == top_a;
  auto extend = [&](const Scaler& s, uint32_t first, uint32_t take) {
    const size_t ncm = s.number_common_moduli;
    PolyRef in = sub_ref(pb, L, logn, 4, first, take);
    PolyRef o = sub_ref(ext, M, logn, 4, first, take);
    o.base += (uint64_t)ncm << logn;
    const ForwardTop fwd{top_a, mc.primes_dev() + ncm};
    rns_scale(*s.rns, logn, in, o, (uint32_t)ncm, (uint32_t)(M - ncm), count * take, st,
              top_a ? &top_a_args : nullptr, fuse_c ? &fwd : nullptr);
    if (first == 0) mark(2);
    NttGeom g{mc.primes_dev() + ncm, (uint32_t)(M - ncm), 0};
    if (fuse_c) ntt_forward_after_top<true>(logn, g, count * take, DstPoly{o}, st, plan_c);
    else ntt_forward_any<true>(logn, g, count * take, SrcPoly{o}, DstPoly{o}, st, plan_c);
  };
  if (same_ext) {
    extend(*ext_lhs, 0, 4);
  } else {
    extend(*ext_lhs, 0, 2);
    extend(*ext_rhs, 2, 2);
  }
  mark(3);
  // D: tensor product fused into the inverse NTT over the extended basis, or
  // (tensor_split) an element-wise product kernel followed by the inverse
  // NTT in place: the separate kernel keeps enough loads in flight to hide
  // their latency, at the cost of one more pass over the products.
  PolyRef prodref = plain_ref(prod, M, logn);
  const uint32_t top_d = top_stages(plan_d, *down, nullptr, (uint32_t)L);
  {
    NttGeom g{mc.primes_dev(), (uint32_t)M, 0};
    const SrcTensor tensor{lref, rref, extref, (uint32_t)ncm_l, (uint32_t)ncm_r};
    if (tensor_split) {
      const uint64_t total = 3 * count * M << logn;
      k_tensor<<<nblocks(total, 256), 256, 0, st>>>(mc.primes_dev(), tensor, prodref, (uint32_t)M, logn, total);
      after_launch("k_tensor");
      if (top_d) ntt_inverse_blocks(logn, g, 3 * count, SrcPolyMont{prodref}, DstPoly{prodref}, st, plan_d);
      else ntt_inverse_any(logn, g, 3 * count, SrcPolyMont{prodref}, DstPoly{prodref}, st, plan_d);
    } else if (top_d) {
      ntt_inverse_blocks(logn, g, 3 * count, tensor, DstPoly{prodref}, st, plan_d);
    } else {
      ntt_inverse_any(logn, g, 3 * count, tensor, DstPoly{prodref}, st, plan_d);
    }
  }
  mark(4);
  // E: scale down by t/Q into the base context (power basis), applying the
  // strided last stages of D's inverse NTT (Montgomery products) on the way.
  PolyRef dnref = plain_ref(dn, L, logn);
  const InverseTop top_d_args{top_d, 1u, mc.primes_dev()};
  // F's strided first stages run in E's epilogue when F's plan has as many as
  // D's: c0 and c1 get them over their own limbs (left in dn for F's block
  // pass), and c2 is expanded there into the digit rows of every key modulus
  // (written to D), so F runs only its block passes.
  const uint32_t bf = plan_f ? plan_f : ntt_block_logn(logn);
  const bool fuse_f = rk && top_d && bf < logn && logn - bf == top_d;
  ForwardTop fwd_e{top_d, bc.primes_dev()};
  if (fuse_f) {
    fwd_e.period = 3;
    fwd_e.take = 2;
    fwd_e.digit_primes = rk->ctx_ksk->primes_dev();
    fwd_e.digit_limbs = (uint32_t)Lk;
    fwd_e.digit_raw = digits_fit(bc.moduli, rk->ctx_ksk->moduli);
    fwd_e.digits = plain_ref(D, Lk, logn);
  }
  rns_scale(*down->rns, logn, prodref, dnref, 0, (uint32_t)L, 3 * count, st, top_d ? &top_d_args : nullptr,
            fuse_f ? &fwd_e : nullptr);
  mark(5);
  NttGeom gb{bc.primes_dev(), (uint32_t)L, 0};
  if (rk) {
    const Context& kc = *rk->ctx_ksk;
    PolyRef dref = plain_ref(D, Lk, logn);
    PolyRef c2 = sub_ref(dn, L, logn, 3, 2, 1);
    PolyRef c01 = sub_ref(dn, L, logn, 3, 0, 2);
    PolyRef oref = plain_ref(dest, L, logn);
    NttGeom gk{kc.primes_dev(), (uint32_t)Lk, 0};
    if (fuse_f) {
      ntt_forward_after_top<true>(logn, gk, count * L, DstPoly{dref}, st, bf);
      ntt_forward_after_top<true>(logn, gb, 2 * count, DstPoly{c01}, DstPoly{oref}, st, bf);
    } else if (bf >= logn && !f_split) {
      // F: digit NTTs and the c0 / c1 NTTs in one launch (Lk == L).
      const uint32_t ndp = (uint32_t)(count * L);
      ntt_fwd_single<true>(logn, gk, count * L + 2 * count, SrcKsF{c2, c01, (uint32_t)L, ndp},
                           DstKsF{dref, oref, ndp}, st);
    } else {
      ntt_forward_any<true>(logn, gk, count * L, SrcDigit{c2, (uint32_t)L, digits_fit(bc.moduli, kc.moduli)},
                            DstPoly{dref}, st, bf);
      ntt_forward_any<true>(logn, gb, 2 * count, SrcPoly{c01}, DstPoly{oref}, st, bf);
    }
    mark(6);
    // G: key inner product added to c0, c1 in place.
    launch_key_mac(bc.primes_dev(), dref, rk->values(0), rk->values(1), dest, 2 * L * N, 0, dest + L * N,
                   2 * L * N, dest, 2 * L * N, (uint32_t)L, (uint32_t)Lk, logn, count, st);
  } else {
    PolyRef o = plain_ref(dest, L, logn);
    ntt_forward_any<true>(logn, gb, 3 * count, SrcPoly{dnref}, DstPoly{o}, st);
    mark(6);
  }
  if (mod_switch) {
    PolyRef in = plain_ref(tmp, L, logn);
    PolyRef o = plain_ref(out, L - 1, logn);
    poly_switch_down_ntt(bc, in, o, count * parts, st);
  }
  mark(7);
}

}  // namespace fheg
