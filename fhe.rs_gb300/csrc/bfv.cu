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
#include <functional>

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
  // into shared memory with asynchronous copies, so every load of the phase
  // is in flight at once instead of what the registers can hold. A square
  // part (l0 r0 or l1 r1) stages half a block of its two operands at a time;
  // the cross term (l0 r1 + l1 r0) a quarter block of its four, so that its
  // two products are summed exactly (below 2 q_j^2 < q_j 2^64) and reduced
  // once, as the unstaged path does.
  template <int LOGN, int T, int E>
  __device__ __forceinline__ void stage(const NttJob& j, const DevPrime& pr, uint32_t base, uint64_t* sm,
                                        uint32_t tid, uint64_t* x) const {
    constexpr uint32_t HALF = 1u << (LOGN - 1), QTR = HALF / 2;
    const uint32_t b = j.poly / 3, part = j.poly % 3;
    if (part != 1) {
      const uint64_t* ra = row(b, part >> 1, j.limb) + base;
      const uint64_t* rb = row(b, 2 + (part >> 1), j.limb) + base;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        for (uint32_t c = tid; c < HALF / 2; c += T) {
          cp_async16(sm + 2 * c, ra + h * HALF + 2 * c);
          cp_async16(sm + HALF + 2 * c, rb + h * HALF + 2 * c);
        }
        cp_async_wait_all();
        __syncthreads();
#pragma unroll
        for (int e = 0; e < E / 2; e++) {
          const uint32_t idx = tid + e * T;
          const uint64_t u = sm[idx], v = sm[HALF + idx];
          x[h * (E / 2) + e] = mont_reduce(__umul64hi(u, v), u * v, pr);
        }
        __syncthreads();
      }
      return;
    }
    const uint64_t* r0 = row(b, 0, j.limb) + base;
    const uint64_t* r1 = row(b, 3, j.limb) + base;
    const uint64_t* r2 = row(b, 1, j.limb) + base;
    const uint64_t* r3 = row(b, 2, j.limb) + base;
#pragma unroll
    for (int qt = 0; qt < 4; qt++) {
      for (uint32_t c = tid; c < QTR / 2; c += T) {
        cp_async16(sm + 2 * c, r0 + qt * QTR + 2 * c);
        cp_async16(sm + QTR + 2 * c, r1 + qt * QTR + 2 * c);
        cp_async16(sm + 2 * QTR + 2 * c, r2 + qt * QTR + 2 * c);
        cp_async16(sm + 3 * QTR + 2 * c, r3 + qt * QTR + 2 * c);
      }
      cp_async_wait_all();
      __syncthreads();
#pragma unroll
      for (int e = 0; e < E / 4; e++) {
        const uint32_t idx = tid + e * T;
        uint64_t hi = 0, lo = 0;
        mac128(hi, lo, sm[idx], sm[QTR + idx]);
        mac128(hi, lo, sm[2 * QTR + idx], sm[3 * QTR + idx]);
        x[qt * (E / 4) + e] = mont_reduce(hi, lo, pr);
      }
      __syncthreads();
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

// Digit d of the base-2^log_base decomposition of a single-limb power-basis
// row (key_switching_key.rs:300-314), lazily reduced into the key modulus
// (rq/mod.rs:525-528): polynomial b * nd + d reads row b.
struct SrcDecompDigit {
  PolyRef rows;  // poly b, limb 0
  uint32_t nd, log_base;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint32_t b = j.poly / nd, d = j.poly % nd;
    const uint64_t x = (rows.at(b, 0)[i] >> (d * log_base)) & ((1ull << log_base) - 1);
    return reduce64_lazy(x, pr);
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    prefetch_l2(rows.at(j.poly / nd, 0) + i);
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
// MAXD > 0 (KB = 1, ndig <= MAXD): every digit and key residue is loaded
// before the first product, so all of a thread's loads are in flight at once.
template <int KB, int MAXD = 0>
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
  if constexpr (MAXD > 0) {
    static_assert(KB == 1, "digits up front take one ciphertext per thread");
    uint64_t x[MAXD], w0[MAXD], w1[MAXD];
    const uint64_t* dp = D + b0 * ndig * dstride + ((uint64_t)j << logn) + i;
#pragma unroll
    for (int d = 0; d < MAXD; d++) {
      if ((uint32_t)d < ndig) {
        w0[d] = __ldg(kp0 + d * kstride);
        w1[d] = __ldg(kp1 + d * kstride);
        x[d] = dp[d * dstride];
      }
    }
#pragma unroll
    for (int d = 0; d < MAXD; d++) {
      if ((uint32_t)d < ndig) {
        mac128(hi0[0], lo0[0], x[d], w0[d]);
        mac128(hi1[0], lo1[0], x[d], w1[d]);
        if (d % 15 == 14) {
          lo0[0] = reduce128(hi0[0], lo0[0], pr);
          hi0[0] = 0;
          lo1[0] = reduce128(hi1[0], lo1[0], pr);
          hi1[0] = 0;
        }
      }
    }
  }
  // The digits of the generic form (MAXD 0): the other forms took theirs above.
  if constexpr (MAXD == 0) {
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
  if (ndig <= 8)
    k_key_mac<1, 8><<<nblocks(total, 256), 256, 0, st>>>(primes, D.base, D.grp_stride, k0, k1, add0, add0_stride,
                                                         add0_e, add1, add1_stride, out, out_stride, ndig, lk, logn,
                                                         batch, total);
  else if (ndig <= 16)
    k_key_mac<1, 16><<<nblocks(total, 256), 256, 0, st>>>(primes, D.base, D.grp_stride, k0, k1, add0, add0_stride,
                                                          add0_e, add1, add1_stride, out, out_stride, ndig, lk, logn,
                                                          batch, total);
  else
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
// Keys below the ciphertext level: the key switch's output lives in the key
// context (Lk > L moduli) and is brought down to the ciphertext context by
// switch_down_to (rq/mod.rs:455-462), i.e. Lk - L successive switch_down
// steps (rq/mod.rs:390-448), each dropping the last modulus with rounding.
// The steps work column by column, so all of them run in one kernel with the
// residues of a coefficient in registers, in the reference's order.

static size_t round32(size_t words) { return (words + 31) & ~(size_t)31; }

void ksk_build_switch_chain(Ksk& k) {
  const size_t Lk = k.ctx_ksk->L(), L = k.ctx_ct->L();
  k.chain.release();
  if (Lk <= L) return;
  const std::vector<uint64_t>& q = k.ctx_ksk->moduli;
  std::vector<uint64_t> t;
  for (size_t m = Lk - 1; m >= L; m--) {
    // The constants of the context with m + 1 moduli (rq/context.rs:66-73,
    // rq/mod.rs:427), for the step that drops q_m.
    t.push_back(q[m]);
    std::vector<uint64_t> inv(m);
    for (size_t i = 0; i < m; i++) inv[i] = invmod(q[m] % q[i], q[i]);
    for (size_t i = 0; i < m; i++) t.push_back(inv[i]);
    for (size_t i = 0; i < m; i++) t.push_back(shoup(inv[i], q[i]));
    for (size_t i = 0; i < m; i++) t.push_back(q[i] - (q[m] / 2) % q[i]);
    if (m == L) break;
  }
  k.chain.alloc(t.size() * 8);
  upload(k.chain.ptr, t.data(), t.size() * 8);
}

// One step (rq/mod.rs:417-438) for residue x (mod q_k) given the dropped
// residue xm (mod q_m) and the step's constants c (see Ksk::chain).
__device__ __forceinline__ uint64_t chain_step(uint64_t x, uint64_t last, const DevPrime& pr, const uint64_t* c,
                                               uint32_t m, uint32_t k) {
  const uint64_t tmp = reduce64_lazy(last, pr) + __ldg(c + 1 + 2 * m + k);
  return mul_shoup(x + 3 * pr.p - tmp, __ldg(c + 1 + k), __ldg(c + 1 + m + k), pr.p);
}

// The steps m = lk-1 .. l on the residues x[0..lk) of one coefficient, held
// in registers (every index static after unrolling).
template <int MAXK>
__device__ __forceinline__ void chain_coeff(uint64_t* x, const DevPrime* primes, const uint64_t* c, uint32_t lk,
                                            uint32_t l) {
#pragma unroll
  for (int m = MAXK - 1; m >= 1; m--) {
    if ((uint32_t)m < lk && (uint32_t)m >= l) {
      const uint64_t qm = __ldg(c);
      const uint64_t last = reduce_once(x[m] + (qm >> 1), qm);
#pragma unroll
      for (int k = 0; k < m; k++) x[k] = chain_step(x[k], last, primes[k], c, (uint32_t)m, (uint32_t)k);
      c += 1 + 3 * m;
    }
  }
}

// `polys` polynomials: in [poly][lk][N] power basis -> out [poly][l][N].
template <int MAXK>
__global__ void k_switch_chain(const DevPrime* primes, const uint64_t* chain, uint32_t lk, uint32_t l, uint32_t logn,
                               PolyRef in, PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t poly = row_of(gid, logn);
  uint64_t x[MAXK];
#pragma unroll
  for (int k = 0; k < MAXK; k++)
    if ((uint32_t)k < lk) x[k] = in.at(poly, k)[i];
  chain_coeff<MAXK>(x, primes, chain, lk, l);
#pragma unroll
  for (int k = 0; k < MAXK; k++)
    if ((uint32_t)k < l) out.at(poly, k)[i] = x[k];
}

// Key contexts of more than 32 moduli: the same steps with the residues
// updated in place in `in`.
__global__ void k_switch_chain_mem(const DevPrime* primes, const uint64_t* chain, uint32_t lk, uint32_t l,
                                   uint32_t logn, PolyRef in, PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t poly = row_of(gid, logn);
  const uint64_t* c = chain;
  for (uint32_t m = lk - 1; m >= l; m--) {
    const uint64_t qm = __ldg(c);
    const uint64_t last = reduce_once(in.at(poly, m)[i] + (qm >> 1), qm);
    for (uint32_t k = 0; k < m; k++) {
      uint64_t* xp = in.at(poly, k) + i;
      *xp = chain_step(*xp, last, primes[k], c, m, k);
    }
    c += 1 + 3 * (uint64_t)m;
    if (m == l) break;
  }
  for (uint32_t k = 0; k < l; k++) out.at(poly, k)[i] = in.at(poly, k)[i];
}

void switch_down_chain(const Ksk& k, PolyRef in, PolyRef out, uint64_t polys, cudaStream_t st) {
  const Context& kc = *k.ctx_ksk;
  const uint32_t lk = (uint32_t)kc.L(), l = (uint32_t)k.ctx_ct->L();
  const uint64_t total = polys << kc.logn;
  if (total == 0 || lk <= l) return;
  const uint64_t* c = k.chain.u64();
  const unsigned blocks = nblocks(total, 256);
  if (lk <= 8) k_switch_chain<8><<<blocks, 256, 0, st>>>(kc.primes_dev(), c, lk, l, kc.logn, in, out, total);
  else if (lk <= 16) k_switch_chain<16><<<blocks, 256, 0, st>>>(kc.primes_dev(), c, lk, l, kc.logn, in, out, total);
  else if (lk <= 32) k_switch_chain<32><<<blocks, 256, 0, st>>>(kc.primes_dev(), c, lk, l, kc.logn, in, out, total);
  else k_switch_chain_mem<<<blocks, 256, 0, st>>>(kc.primes_dev(), c, lk, l, kc.logn, in, out, total);
  after_launch("k_switch_chain");
}

// Destination of the last forward NTT of a switched-down key switch: part
// `poly & 1` of ciphertext `poly >> 1`, plus the ciphertext part it is added
// to (add0 optionally read through the substitution of exponent add0_e).
struct DstAddParts {
  uint64_t* out;
  uint64_t out_stride;
  const uint64_t* add0;
  uint64_t add0_stride, add0_e;
  const uint64_t* add1;
  uint64_t add1_stride;
  uint32_t L, logn;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime& pr, uint32_t i, uint64_t v) const {
    const uint64_t b = j.poly >> 1;
    const uint32_t part = j.poly & 1;
    uint64_t a = 0;
    if (part == 0) {
      if (add0) a = add0[b * add0_stride + ((uint64_t)j.limb << logn) + (add0_e ? gather_index(i, add0_e, logn) : i)];
    } else if (add1) {
      a = add1[b * add1_stride + ((uint64_t)j.limb << logn) + i];
    }
    out[b * out_stride + ((uint64_t)(part * L + j.limb) << logn) + i] = add_mod(v, a, pr.p);
  }
};

// Forward NTT of `inplace` (reduced) whose final values go to `dst`; a
// two-pass plan runs its strided pass in place first.
template <class Dst>
void ntt_forward_into(uint32_t logn, NttGeom g, uint64_t polys, PolyRef inplace, Dst dst, cudaStream_t st) {
  const uint32_t bl = ntt_block_logn(logn);
  if (bl >= logn || logn < 13) {
    g.s1 = 0;
    ntt_fwd_single<true>(logn, g, polys, SrcPoly{inplace}, dst, st);
    return;
  }
  if (bl == 12 && ntt_cluster_enabled(logn) &&
      launch_fwd_cluster<12, true>(g, logn - bl, polys, SrcPoly{inplace}, dst, st))
    return;
  launch_fwd_top(logn - bl, g, bl, polys, SrcPoly{inplace}, DstPoly{inplace}, st);
  ntt_forward_after_top<true>(logn, g, polys, DstPoly{inplace}, dst, st, bl);
}

// The key context's (c0, c1) of `batch` key switches in `ks` ([batch][2][Lk][N],
// Ntt; overwritten) into the power basis, down to the ciphertext context
// (`sd`, [batch][2][L][N]), back to Ntt, plus add0 / add1, into out.
static void finish_switch_down(const Ksk& k, uint64_t* ks, uint64_t* sd, uint64_t batch, const uint64_t* add0,
                               uint64_t add0_poly_stride, uint64_t add0_exponent, const uint64_t* add1,
                               uint64_t add1_poly_stride, uint64_t* out, uint64_t out_poly_stride, cudaStream_t st) {
  const Context& kc = *k.ctx_ksk;
  const Context& cc = *k.ctx_ct;
  const uint32_t logn = kc.logn;
  PolyRef ksref = plain_ref(ks, kc.L(), logn);
  PolyRef sdref = plain_ref(sd, cc.L(), logn);
  ntt_backward(kc, ksref, ksref, 2 * batch, st);
  switch_down_chain(k, ksref, sdref, 2 * batch, st);
  NttGeom g{cc.primes_dev(), (uint32_t)cc.L(), 0};
  DstAddParts dst{out, out_poly_stride, add0, add0_poly_stride, add0_exponent, add1, add1_poly_stride,
                  (uint32_t)cc.L(), logn};
  ntt_forward_into(logn, g, 2 * batch, sdref, dst, st);
}

// ---------------------------------------------------------------------------
// Key switching (key_switching_key.rs:214-289) on digits in the power basis.

size_t key_switch_scratch_words(const Ksk& k, uint64_t batch) {
  const size_t Lk = k.ctx_ksk->L(), L = k.ctx_ct->L(), N = k.ctx_ct->N();
  size_t w = round32(batch * k.count * Lk * N);
  if (k.switches_down()) w += round32(batch * 2 * Lk * N) + round32(batch * 2 * L * N);
  return w;
}

void key_switch(const Ksk& k, PolyRef digits, uint64_t batch, const uint64_t* add0, uint64_t add0_poly_stride,
                uint64_t add0_exponent, const uint64_t* add1, uint64_t add1_poly_stride, uint64_t* out,
                uint64_t out_poly_stride, uint64_t* D, cudaStream_t st) {
  const Context& kc = *k.ctx_ksk;
  const size_t Lk = kc.L(), nd = k.count, N = kc.N();
  const uint32_t logn = kc.logn;
  PolyRef dref = plain_ref(D, Lk, logn);
  NttGeom g{kc.primes_dev(), (uint32_t)Lk, 0};
  // Every digit in every key modulus (rq/mod.rs:518-540), reduced output.
  if (k.log_base)
    ntt_forward_any<true>(logn, g, batch * nd, SrcDecompDigit{digits, (uint32_t)nd, k.log_base}, DstPoly{dref}, st);
  else
    ntt_forward_any<true>(logn, g, batch * nd,
                          SrcDigit{digits, (uint32_t)nd, digits_fit(k.ctx_ct->moduli, kc.moduli)}, DstPoly{dref},
                          st);
  if (!k.switches_down()) {
    launch_key_mac(kc.primes_dev(), dref, k.values(0), k.values(1), add0, add0_poly_stride, add0_exponent, add1,
                   add1_poly_stride, out, out_poly_stride, (uint32_t)nd, (uint32_t)Lk, logn, batch, st);
    return;
  }
  // relinearization_key.rs:84-92, galois_key.rs:113-120: the sums in the key
  // context, switched down, then added.
  uint64_t* ks = D + round32(batch * nd * Lk * N);
  uint64_t* sd = ks + round32(batch * 2 * Lk * N);
  launch_key_mac(kc.primes_dev(), dref, k.values(0), k.values(1), nullptr, 0, 0, nullptr, 0, ks, 2 * Lk * N,
                 (uint32_t)nd, (uint32_t)Lk, logn, batch, st);
  finish_switch_down(k, ks, sd, batch, add0, add0_poly_stride, add0_exponent, add1, add1_poly_stride, out,
                     out_poly_stride, st);
}

void relinearize(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st) {
  const Context& c = *rk.ctx_ct;
  const size_t L = c.L(), N = c.N();
  if (count == 0) return;
  const size_t d_words = key_switch_scratch_words(rk, count);
  ws.reserve((round32(count * L * N) + d_words) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(count * L * N, &off);
  uint64_t* D = ws.take(d_words, &off);
  // relinearization_key.rs:81: c2 into the power basis.
  PolyRef src = sub_ref(const_cast<uint64_t*>(ct3), L, c.logn, 3, 2, 1);
  PolyRef dst = plain_ref(digits, L, c.logn);
  ntt_backward(c, src, dst, count, st);
  // relinearization_key.rs:82-95: key switch, then add to c0 and c1.
  key_switch(rk, dst, count, ct3, 3 * L * N, 0, ct3 + L * N, 3 * L * N, out, 2 * L * N, D, st);
}

// Relinearization with caller-provided scratch: `digits` holds count*L*N
// words and `D` key_switch_scratch_words(rk, count) words. Same computation
// as relinearize().
void relinearize_scratch(const Ksk& rk, const uint64_t* ct3, uint64_t* out, uint64_t count, uint64_t* digits,
                         uint64_t* D, cudaStream_t st) {
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
  const Context& c = *gk.ctx_ct;
  const size_t L = c.L(), N = c.N();
  const uint64_t e = exponent % (2 * N);
  if ((e & 1) == 0) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
  if (count == 0) return;
  const size_t d_words = key_switch_scratch_words(gk, count);
  ws.reserve((round32(count * L * N) + d_words) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(count * L * N, &off);
  uint64_t* D = ws.take(d_words, &off);
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

// 16-byte size: the uint4 job table follows `count` descriptors in memory.
struct alignas(16) RotDesc {
  const uint64_t* ct;     // [2][L][N] Ntt
  uint64_t* out;          // [2][L][N] Ntt
  uint64_t* digits;       // [L][N] scratch: substituted c1 in the power basis
  uint64_t* D;            // [L digits][Lk limbs][N] scratch: digit NTTs
  const uint64_t* k0;     // [L][Lk][N] key values, part 0
  const uint64_t* k1;     // part 1
  // Keys below the ciphertext level (Lk > L): the key-context sums [2][Lk][N]
  // (then their power basis), their switch-down [2][L][N] (then its Ntt)
  // and the switch-down constants; null otherwise.
  uint64_t* ks;
  uint64_t* sd;
  const uint64_t* chain;
  uint64_t e;             // substitution exponent mod 2N
  uint32_t L, Lk;
  uint32_t nd;            // digits: L, or those of a base-2^log_base decomposition
  uint32_t log_base;      // 0 for RNS digits
};
static_assert(sizeof(RotDesc) % 16 == 0, "the job table after the descriptors needs 16-byte alignment");

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
    const RotDesc& r = d[j.poly];
    if (r.log_base)
      return reduce64_lazy((r.digits[i] >> (j.aux * r.log_base)) & ((1ull << r.log_base) - 1), pr);
    return reduce64_lazy(r.digits[((uint64_t)j.aux << logn) + i], pr);
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
    return r.D + ((uint64_t)(j.aux * r.Lk + j.limb) << logn) + i;
  }
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    *at(j, i) = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const { return *at(j, i); }
};

// G: out0 = substitute(ct0) + sum_d D[d] * k0[d], out1 = sum_d D[d] * k1[d]
// for row (poly, limb) = rows[blockIdx.y]; exact sums reduced once. Requests
// whose key switches down write the bare sums (key context) to ks instead.
__global__ void k_rot_mac(const DevPrime* primes, const RotDesc* d, const uint2* rows, uint32_t logn) {
  const uint2 row = rows[blockIdx.y];
  const RotDesc& r = d[row.x];
  const uint32_t j = row.y;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << logn)) return;
  const DevPrime pr = primes[j];
  const uint64_t plane = (uint64_t)r.Lk << logn;
  uint64_t* const o = r.ks ? r.ks : r.out;
  uint64_t lo0 = r.ks ? 0 : r.ct[((uint64_t)j << logn) + gather_index(i, r.e, logn)], hi0 = 0, lo1 = 0, hi1 = 0;
  for (uint32_t dd = 0; dd < r.nd; dd++) {
    const uint64_t off = ((uint64_t)(dd * r.Lk + j) << logn) + i;
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
  o[((uint64_t)j << logn) + i] = reduce128(hi0, lo0, pr);
  o[plane + ((uint64_t)j << logn) + i] = reduce128(hi1, lo1, pr);
}

// Switch-down of the requests whose key lies below their level
// (galois_key.rs:113-120): part `aux` of request `poly`, limb `limb`, of the
// key-context sums (inverse NTT in place) and of the switched-down result
// (forward NTT in place).
struct RotKs {
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ uint64_t* at(const NttJob& j, uint32_t i) const {
    const RotDesc& r = d[j.poly];
    return r.ks + ((uint64_t)(j.aux * r.Lk + j.limb) << logn) + i;
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return *at(j, i);
  }
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    *at(j, i) = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const { return *at(j, i); }
};

struct RotSd {
  const RotDesc* d;
  uint32_t logn;
  __device__ __forceinline__ uint64_t* at(const NttJob& j, uint32_t i) const {
    const RotDesc& r = d[j.poly];
    return r.sd + ((uint64_t)(j.aux * r.L + j.limb) << logn) + i;
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return *at(j, i);
  }
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    *at(j, i) = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const { return *at(j, i); }
};

// The switch-down chain of part jobs[blockIdx.y] = (request, part): its Lk
// power-basis residues of each coefficient down to L (moduli are a prefix of
// one chain, so limb k of every request uses primes[k]).
template <int MAXK>
__global__ void k_rot_chain(const DevPrime* primes, const RotDesc* d, const uint2* jobs, uint32_t logn) {
  const uint2 job = jobs[blockIdx.y];
  const RotDesc& r = d[job.x];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << logn)) return;
  const uint64_t* in = r.ks + ((uint64_t)(job.y * r.Lk) << logn) + i;
  uint64_t* out = r.sd + ((uint64_t)(job.y * r.L) << logn) + i;
  uint64_t x[MAXK];
#pragma unroll
  for (int k = 0; k < MAXK; k++)
    if ((uint32_t)k < r.Lk) x[k] = in[(uint64_t)k << logn];
  chain_coeff<MAXK>(x, primes, r.chain, r.Lk, r.L);
#pragma unroll
  for (int k = 0; k < MAXK; k++)
    if ((uint32_t)k < r.L) out[(uint64_t)k << logn] = x[k];
}

// Last step of those requests: out0 = sd0 + substitute(ct0), out1 = sd1, for
// row rows[blockIdx.y] = (request, part * L + limb).
__global__ void k_rot_add(const DevPrime* primes, const RotDesc* d, const uint2* rows, uint32_t logn) {
  const uint2 row = rows[blockIdx.y];
  const RotDesc& r = d[row.x];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1u << logn)) return;
  const uint32_t part = row.y >= r.L ? 1 : 0, j = row.y - part * r.L;
  const uint64_t at = ((uint64_t)row.y << logn) + i;
  uint64_t v = r.sd[at];
  if (part == 0) v = add_mod(v, r.ct[((uint64_t)j << logn) + gather_index(i, r.e, logn)], primes[j].p);
  r.out[at] = v;
}

namespace {
// Scratch words and table entries of a ragged batch.
struct RotCounts {
  size_t digit_words = 0, d_words = 0, ks_words = 0, sd_words = 0;
  size_t n_r1 = 0, n_f = 0, n_inv = 0, n_fwd = 0, n_rows = 0, n_chain = 0, n_add = 0;
  uint32_t max_lk = 0;
  size_t table_words(size_t count) const {
    return (count * sizeof(RotDesc) + (n_r1 + n_f + n_inv + n_fwd) * sizeof(uint4) +
            (n_rows + n_chain + n_add) * sizeof(uint2)) / 8 + 8;
  }
};

RotCounts rot_counts(const RotRequest* req, size_t count) {
  RotCounts c;
  for (size_t b = 0; b < count; b++) {
    const Ksk& k = *req[b].key;
    const size_t L = k.ctx_ct->L(), Lk = k.ctx_ksk->L(), N = k.ctx_ct->N(), nd = k.count;
    c.digit_words += L * N;
    c.d_words += nd * Lk * N;
    c.n_r1 += L;
    c.n_f += nd * Lk;
    c.n_rows += Lk;
    if (k.switches_down()) {
      c.ks_words += 2 * Lk * N;
      c.sd_words += 2 * L * N;
      c.n_inv += 2 * Lk;
      c.n_fwd += 2 * L;
      c.n_chain += 2;
      c.n_add += 2 * L;
      c.max_lk = std::max(c.max_lk, (uint32_t)Lk);
    }
  }
  return c;
}
}  // namespace

size_t galois_batch_scratch_bytes(const RotRequest* req, size_t count) {
  const RotCounts c = rot_counts(req, count);
  return (c.digit_words + c.d_words + c.ks_words + c.sd_words + c.table_words(count) + 128 + 6 * 32) * 8;
}

void validate_rot_requests(const Params& par, const RotRequest* req, size_t count) {
  const size_t N = par.degree;
  for (size_t b = 0; b < count; b++) {
    const Ksk& k = *req[b].key;
    if (k.par != &par) throw Error(FHEG_ERR_KEY_MISMATCH, "all keys of a batch must share the parameters");
    if ((req[b].exponent % (2 * N)) % 2 == 0)
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "The exponent should be odd modulo 2 * degree");
    if (k.switches_down() && k.ctx_ksk->L() > 32)
      throw Error(FHEG_ERR_UNSUPPORTED, "batched rotations switch down from key contexts of at most 32 moduli");
  }
}

// The device tables and scratch of one ragged batch, ready to launch.
struct RotBatchPlan {
  const Params* par = nullptr;
  RotCounts cnt;
  const RotDesc* d_desc = nullptr;
  const uint4* d_jobs = nullptr;
  const uint2* d_rows = nullptr;
};

static void launch_rot_batch(const RotBatchPlan& pl, cudaStream_t st);

// Builds the batch's tables in `ws` (scratch included) and uploads them on
// `st`; the copies from host memory complete before this returns.
static RotBatchPlan prepare_rot_batch(const Params& par, const RotRequest* req, size_t count, Workspace& ws,
                                     cudaStream_t st) {
  validate_rot_requests(par, req, count);
  const size_t N = par.ctx(0)->N();
  // Scratch and tables.
  const RotCounts cnt = rot_counts(req, count);
  const size_t table_words = cnt.table_words(count);
  ws.reserve((cnt.digit_words + cnt.d_words + cnt.ks_words + cnt.sd_words + table_words + 128 + 6 * 32) * 8);
  size_t off = 0;
  uint64_t* digits = ws.take(cnt.digit_words, &off);
  uint64_t* D = ws.take(cnt.d_words, &off);
  uint64_t* KS = ws.take(cnt.ks_words, &off);
  uint64_t* SD = ws.take(cnt.sd_words, &off);
  uint64_t* tables = ws.take(table_words, &off);
  std::vector<RotDesc> desc(count);
  std::vector<uint4> jobs;
  jobs.reserve(cnt.n_r1 + cnt.n_f + cnt.n_inv + cnt.n_fwd);
  std::vector<uint2> rows;
  rows.reserve(cnt.n_rows + cnt.n_chain + cnt.n_add);
  size_t dpos = 0, Dpos = 0, kpos = 0, spos = 0;
  for (size_t b = 0; b < count; b++) {
    const Ksk& k = *req[b].key;
    const uint32_t L = (uint32_t)k.ctx_ct->L(), Lk = (uint32_t)k.ctx_ksk->L();
    RotDesc& r = desc[b];
    r.ct = req[b].ct;
    r.out = req[b].out;
    r.digits = digits + dpos;
    r.D = D + Dpos;
    r.k0 = k.values(0);
    r.k1 = k.values(1);
    r.ks = r.sd = nullptr;
    r.chain = nullptr;
    if (k.switches_down()) {
      r.ks = KS + kpos;
      r.sd = SD + spos;
      r.chain = k.chain.u64();
      kpos += (size_t)2 * Lk * N;
      spos += (size_t)2 * L * N;
    }
    r.e = req[b].exponent % (2 * N);
    r.L = L;
    r.Lk = Lk;
    r.nd = (uint32_t)k.count;
    r.log_base = k.log_base;
    dpos += (size_t)L * N;
    Dpos += (size_t)r.nd * Lk * N;
    for (uint32_t i = 0; i < L; i++) jobs.push_back(make_uint4((uint32_t)b, i, 0, 0));
  }
  for (size_t b = 0; b < count; b++)
    for (uint32_t dd = 0; dd < desc[b].nd; dd++)
      for (uint32_t j = 0; j < desc[b].Lk; j++) jobs.push_back(make_uint4((uint32_t)b, j, dd, 0));
  for (size_t b = 0; b < count; b++)
    if (desc[b].ks)
      for (uint32_t part = 0; part < 2; part++)
        for (uint32_t j = 0; j < desc[b].Lk; j++) jobs.push_back(make_uint4((uint32_t)b, j, part, 0));
  for (size_t b = 0; b < count; b++)
    if (desc[b].ks)
      for (uint32_t part = 0; part < 2; part++)
        for (uint32_t j = 0; j < desc[b].L; j++) jobs.push_back(make_uint4((uint32_t)b, j, part, 0));
  for (size_t b = 0; b < count; b++)
    for (uint32_t j = 0; j < desc[b].Lk; j++) rows.push_back(make_uint2((uint32_t)b, j));
  for (size_t b = 0; b < count; b++)
    if (desc[b].ks)
      for (uint32_t part = 0; part < 2; part++) rows.push_back(make_uint2((uint32_t)b, part));
  for (size_t b = 0; b < count; b++)
    if (desc[b].ks)
      for (uint32_t j = 0; j < 2 * desc[b].L; j++) rows.push_back(make_uint2((uint32_t)b, j));
  // Upload the tables (pageable source: the copy completes before return).
  uint8_t* tb = reinterpret_cast<uint8_t*>(tables);  // 256-byte aligned (Workspace::take)
  RotDesc* d_desc = reinterpret_cast<RotDesc*>(tb);
  uint4* d_jobs = reinterpret_cast<uint4*>(tb + count * sizeof(RotDesc));
  uint2* d_rows = reinterpret_cast<uint2*>(tb + count * sizeof(RotDesc) + jobs.size() * sizeof(uint4));
  check_cuda(cudaMemcpyAsync(d_desc, desc.data(), count * sizeof(RotDesc), cudaMemcpyHostToDevice, st), "H2D");
  check_cuda(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(uint4), cudaMemcpyHostToDevice, st), "H2D");
  check_cuda(cudaMemcpyAsync(d_rows, rows.data(), rows.size() * sizeof(uint2), cudaMemcpyHostToDevice, st), "H2D");
  RotBatchPlan pl;
  pl.par = &par;
  pl.cnt = cnt;
  pl.d_desc = d_desc;
  pl.d_jobs = d_jobs;
  pl.d_rows = d_rows;
  return pl;
}

// The launches of a prepared batch (capturable: no host memory is read).
static void launch_rot_batch(const RotBatchPlan& pl, cudaStream_t st) {
  const Context& top = *pl.par->ctx(0);
  const size_t N = top.N();
  const uint32_t logn = top.logn;
  const RotCounts& cnt = pl.cnt;
  const RotDesc* d_desc = pl.d_desc;
  const uint4* d_jobs = pl.d_jobs;
  const uint2* d_rows = pl.d_rows;
  // R1: substituted c1 into the power basis.
  NttGeom g1{top.primes_dev(), 1, 0, d_jobs};
  ntt_inverse_any(logn, g1, cnt.n_r1, SrcRotSubst{d_desc, logn}, DstRotDigits{d_desc, logn}, st);
  // F: every digit in every key limb.
  NttGeom g2{top.primes_dev(), 1, 0, d_jobs + cnt.n_r1};
  ntt_forward_any<true>(logn, g2, cnt.n_f, SrcRotDigit{d_desc, logn}, DstRotD{d_desc, logn}, st);
  // G: inner products and the substituted c0.
  const unsigned gx = (unsigned)((N + 255) / 256);
  k_rot_mac<<<dim3(gx, (unsigned)cnt.n_rows), 256, 0, st>>>(top.primes_dev(), d_desc, d_rows, logn);
  after_launch("k_rot_mac");
  if (cnt.n_chain == 0) return;
  // Requests with keys below their level: the sums into the power basis, down
  // to the ciphertext context, back to Ntt, plus the substituted c0.
  NttGeom g3{top.primes_dev(), 1, 0, d_jobs + cnt.n_r1 + cnt.n_f};
  ntt_inverse_any(logn, g3, cnt.n_inv, RotKs{d_desc, logn}, RotKs{d_desc, logn}, st);
  const uint2* d_chain = d_rows + cnt.n_rows;
  const dim3 gc(gx, (unsigned)cnt.n_chain);
  if (cnt.max_lk <= 8) k_rot_chain<8><<<gc, 256, 0, st>>>(top.primes_dev(), d_desc, d_chain, logn);
  else if (cnt.max_lk <= 16) k_rot_chain<16><<<gc, 256, 0, st>>>(top.primes_dev(), d_desc, d_chain, logn);
  else k_rot_chain<32><<<gc, 256, 0, st>>>(top.primes_dev(), d_desc, d_chain, logn);
  after_launch("k_rot_chain");
  NttGeom g4{top.primes_dev(), 1, 0, d_jobs + cnt.n_r1 + cnt.n_f + cnt.n_inv};
  ntt_forward_any<true>(logn, g4, cnt.n_fwd, RotSd{d_desc, logn}, RotSd{d_desc, logn}, st);
  k_rot_add<<<dim3(gx, (unsigned)cnt.n_add), 256, 0, st>>>(top.primes_dev(), d_desc, d_chain + cnt.n_chain, logn);
  after_launch("k_rot_add");
}

void galois_relinearize_batch(const Params& par, const RotRequest* req, size_t count, Workspace& ws,
                              cudaStream_t st) {
  if (count == 0) return;
  launch_rot_batch(prepare_rot_batch(par, req, count, ws, st), st);
}

std::function<void(cudaStream_t)> prepare_galois_batch(const Params& par, const RotRequest* req, size_t count,
                                                       Workspace& ws, cudaStream_t st) {
  if (count == 0) return [](cudaStream_t) {};
  const RotBatchPlan pl = prepare_rot_batch(par, req, count, ws, st);
  check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return [pl](cudaStream_t s) { launch_rot_batch(pl, s); };
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
  m->rk = &rk;
  return m;
}

size_t Multiplicator::scratch_bytes(uint64_t count) const {
  const size_t L = base->L(), M = mul->L(), N = base->N();
  const size_t Lk = rk ? rk->ctx_ksk->L() : 0;
  const bool down = rk && rk->switches_down();
  const size_t d_words = !rk ? 0 : rk->log_base ? key_switch_scratch_words(*rk, count) : count * L * Lk * N;
  const size_t words = count * 4 * L * N + count * 4 * M * N + count * 3 * M * N + count * 3 * L * N + d_words +
                       (mod_switch ? count * out_parts() * L * N : 0) +
                       (down ? count * 2 * Lk * N + count * 2 * L * N : 0) + 8 * 32;
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
  const bool ks_down = rk && rk->switches_down();
  // Decomposition keys (single-modulus contexts) take the generic key switch
  // on c2 in the power basis.
  const bool ks_decomp = rk && rk->log_base;
  const size_t w_pb = count * 4 * L * N, w_ext = count * 4 * M * N, w_prod = count * 3 * M * N,
               w_down = count * 3 * L * N,
               w_d = !rk ? 0 : ks_decomp ? key_switch_scratch_words(*rk, count) : count * L * Lk * N,
               w_tmp = mod_switch ? count * parts * L * N : 0, w_ks = ks_down ? count * 2 * Lk * N : 0,
               w_sd = ks_down ? count * 2 * L * N : 0;
  ws.reserve(scratch_bytes(count));
  size_t off = 0;
  uint64_t* pb = ws.take(w_pb, &off);
  uint64_t* ext = ws.take(w_ext, &off);
  uint64_t* prod = ws.take(w_prod, &off);
  uint64_t* dn = ws.take(w_down, &off);
  uint64_t* D = ws.take(w_d, &off);
  uint64_t* tmp = ws.take(w_tmp, &off);
  uint64_t* ks = ws.take(w_ks, &off);
  uint64_t* sd = ws.take(w_sd, &off);
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
  const bool fuse_f = rk && !ks_decomp && top_d && bf < logn && logn - bf == top_d;
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
    if (ks_decomp) {
      // mul.rs:196-210 with key_switching_key.rs:292-329: c0, c1 into Ntt;
      // G below adds the decomposed key switch of c2.
      ntt_forward_any<true>(logn, gb, 2 * count, SrcPoly{c01}, DstPoly{oref}, st, bf);
    } else if (fuse_f) {
      ntt_forward_after_top<true>(logn, gk, count * L, DstPoly{dref}, st, bf);
      ntt_forward_after_top<true>(logn, gb, 2 * count, DstPoly{c01}, DstPoly{oref}, st, bf);
    } else if (bf >= logn && !f_split && !ks_down) {
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
    if (ks_decomp) {
      // G: digit NTTs and the key inner product, added to c0, c1 in place.
      key_switch(*rk, c2, count, dest, 2 * L * N, 0, dest + L * N, 2 * L * N, dest, 2 * L * N, D, st);
    } else if (!ks_down) {
      // G: key inner product added to c0, c1 in place.
      launch_key_mac(bc.primes_dev(), dref, rk->values(0), rk->values(1), dest, 2 * L * N, 0, dest + L * N,
                     2 * L * N, dest, 2 * L * N, (uint32_t)L, (uint32_t)Lk, logn, count, st);
    } else {
      // G with a key below the multiplication level (mul.rs:199-206): the
      // inner product in the key context, switched down to the ciphertext
      // context and added to c0, c1.
      launch_key_mac(kc.primes_dev(), dref, rk->values(0), rk->values(1), nullptr, 0, 0, nullptr, 0, ks, 2 * Lk * N,
                     (uint32_t)L, (uint32_t)Lk, logn, count, st);
      finish_switch_down(*rk, ks, sd, count, dest, 2 * L * N, 0, dest + L * N, 2 * L * N, dest, 2 * L * N, st);
    }
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
