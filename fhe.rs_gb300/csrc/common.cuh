// Device-side modular arithmetic and shared structures for the GB300
// RNS-BFV kernels. All arithmetic is exact u64 residue arithmetic for primes
// below 2^62, as in fhe-math/src/zq/mod.rs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "host_math.hpp"
#include "fheg.h"

namespace fheg {

// Per-prime constants and twiddle tables resident on the device. One entry
// per modulus of a context; kernels index it by limb.
struct DevPrime {
  uint64_t p;           // modulus, < 2^62
  uint64_t p2;          // 2p
  uint64_t bhi, blo;    // floor(2^128 / p), the Barrett constant of zq/mod.rs:83-98
  uint64_t ninv;        // N^-1 mod p
  uint64_t ninv_shoup;  // Shoup companion of ninv
  uint64_t pinv;        // -p^-1 mod 2^64 (Montgomery reduction)
  uint64_t ninv_mont;   // N^-1 * 2^64 mod p: final scale of an inverse NTT of Montgomery products
  uint64_t ninv_mont_shoup;
  // The last inverse stage's twiddle zetas_inv[N - 2] times the final scale
  // (N^-1, or N^-1 * 2^64 for Montgomery inputs), with Shoup companions: the
  // strided inverse pass folds the scaling into that stage's products.
  uint64_t zlast_ninv, zlast_ninv_shoup;
  uint64_t zlast_ninv_mont, zlast_ninv_mont_shoup;
  // Twiddle tables of native.rs:35-73, each entry paired with its Shoup
  // companion so one 16-byte load fetches both: tw[i] = (omegas[i],
  // omegas_shoup[i]), itw[i] = (zetas_inv[i], zetas_inv_shoup[i]).
  const ulonglong2* tw;
  const ulonglong2* itw;
};

// Counts every kernel launch issued by the library (reported by benchmarks).
extern std::atomic<uint64_t> g_launches;

// NTT plan: the block size (log2) used for transforms of 2^logn residues. A
// value >= logn runs the single-pass kernel; a smaller one (12, 13 or 14,
// with logn - bl <= 4) runs a strided pass plus 2^(logn - bl) blocks.
uint32_t ntt_block_logn(uint32_t logn);
// Validates and installs a plan entry (FHEG_ERR_INVALID_ARGUMENT otherwise).
void set_ntt_block_logn(uint32_t logn, uint32_t block_logn);
bool ntt_plan_valid(uint32_t logn, uint32_t block_logn);
// Whether the block kernels prefetch the next CTA's input into L2
// (fheg_ntt_prefetch_set; on by default).
bool ntt_prefetch_enabled();
void set_ntt_prefetch(bool on);
// The valid block sizes for 2^logn, ascending.
std::vector<uint32_t> ntt_plans(uint32_t logn);
// Whether two-pass plans with 2^12-residue blocks run instead as one pass on
// clusters of 2^(logn - 12) CTAs exchanging through distributed shared
// memory (fheg_ntt_cluster_set).
bool ntt_cluster_enabled(uint32_t logn);
void set_ntt_cluster(uint32_t logn, bool on);

inline void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(10 /*FHEG_ERR_CUDA*/, std::string(what) + ": " + cudaGetErrorString(e));
}

// Checks the launch that was just issued and counts it.
inline void after_launch(const char* what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  check_cuda(cudaGetLastError(), what);
}

// Generalised polynomial batch addressing used by the kernels: polynomial
// `poly` lives at base + (poly / grp) * grp_stride + (poly % grp) * poly_stride,
// limb l at + (l << logn).
struct PolyRef {
  uint64_t* base;
  uint64_t grp_stride;
  uint64_t poly_stride;
  uint32_t grp;
  uint32_t logn;
  __host__ __device__ __forceinline__ uint64_t* at(uint32_t poly, uint32_t limb) const {
    return base + (uint64_t)(poly / grp) * grp_stride + (uint64_t)(poly % grp) * poly_stride +
           ((uint64_t)limb << logn);
  }
};

// Row (one limb of one polynomial) of element `gid` of a [rows][2^logn]
// array. Rows fit in 32 bits (2^32 rows of at least 8 residues exceed any
// device memory), so splitting a row into (polynomial, limb) is a 32-bit
// division by the limb count rather than a much longer 64-bit one.
__device__ __forceinline__ uint32_t row_of(uint64_t gid, uint32_t logn) { return (uint32_t)(gid >> logn); }

inline PolyRef plain_ref(uint64_t* base, size_t limbs, uint32_t logn) {
  PolyRef r;
  r.base = base;
  r.grp = 1;
  r.poly_stride = (uint64_t)limbs << logn;
  r.grp_stride = r.poly_stride;
  r.logn = logn;
  return r;
}

// Polynomials `first .. first+take-1` of every group of `grp` polynomials
// with `limbs` limbs each.
inline PolyRef sub_ref(uint64_t* base, size_t limbs, uint32_t logn, uint32_t grp, uint32_t first,
                       uint32_t take) {
  PolyRef r;
  r.poly_stride = (uint64_t)limbs << logn;
  r.grp_stride = r.poly_stride * grp;
  r.base = base + r.poly_stride * first;
  r.grp = take;
  r.logn = logn;
  return r;
}

// ---------------------------------------------------------------------------
// Device arithmetic

// zq/mod.rs:224-234 `lazy_mul_shoup`: a * b mod p in [0, 2p) for any a < 2^64,
// with b_shoup = floor(b * 2^64 / p). (Measured against hand-written 32-bit
// PTX sequences on GB300, this form issues the fewest instructions.)
__device__ __forceinline__ uint64_t mul_shoup_lazy(uint64_t a, uint64_t b, uint64_t b_shoup, uint64_t p) {
  return a * b - __umul64hi(a, b_shoup) * p;
}

// Exact multiply-accumulate into a 128-bit accumulator (hi:lo) += a * b.
// The caller guarantees the sum stays below 2^128.
__device__ __forceinline__ void mac128(uint64_t& hi, uint64_t& lo, uint64_t a, uint64_t b) {
  asm("{\n\t"
      ".reg .u32 a0, a1, b0, b1, w0, w1, w2, w3;\n\t"
      "mov.b64 {a0, a1}, %2;\n\t"
      "mov.b64 {b0, b1}, %3;\n\t"
      "mov.b64 {w0, w1}, %1;\n\t"
      "mov.b64 {w2, w3}, %0;\n\t"
      "mad.lo.cc.u32 w0, a0, b0, w0;\n\t"
      "madc.hi.cc.u32 w1, a0, b0, w1;\n\t"
      "madc.lo.cc.u32 w2, a1, b1, w2;\n\t"
      "madc.hi.u32 w3, a1, b1, w3;\n\t"
      "mad.lo.cc.u32 w1, a0, b1, w1;\n\t"
      "madc.hi.cc.u32 w2, a0, b1, w2;\n\t"
      "addc.u32 w3, w3, 0;\n\t"
      "mad.lo.cc.u32 w1, a1, b0, w1;\n\t"
      "madc.hi.cc.u32 w2, a1, b0, w2;\n\t"
      "addc.u32 w3, w3, 0;\n\t"
      "mov.b64 %1, {w0, w1};\n\t"
      "mov.b64 %0, {w2, w3};\n\t"
      "}"
      : "+l"(hi), "+l"(lo)
      : "l"(a), "l"(b));
}

// w[0..6) (192 bits, 32-bit words) += x * (bhi:blo) for x < 2^64, b < 2^128.
// The caller guarantees the sum stays below 2^192.
__device__ __forceinline__ void mac192(uint32_t* w, uint64_t x, uint64_t blo, uint64_t bhi) {
  asm("{\n\t"
      ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
      "mov.b64 {x0, x1}, %6;\n\t"
      "mov.b64 {b0, b1}, %7;\n\t"
      "mov.b64 {b2, b3}, %8;\n\t"
      "mad.lo.cc.u32 %0, x0, b0, %0;\n\t"
      "madc.lo.cc.u32 %1, x0, b1, %1;\n\t"
      "madc.lo.cc.u32 %2, x0, b2, %2;\n\t"
      "madc.lo.cc.u32 %3, x0, b3, %3;\n\t"
      "addc.cc.u32 %4, %4, 0;\n\t"
      "addc.u32 %5, %5, 0;\n\t"
      "mad.hi.cc.u32 %1, x0, b0, %1;\n\t"
      "madc.hi.cc.u32 %2, x0, b1, %2;\n\t"
      "madc.hi.cc.u32 %3, x0, b2, %3;\n\t"
      "madc.hi.cc.u32 %4, x0, b3, %4;\n\t"
      "addc.u32 %5, %5, 0;\n\t"
      "mad.lo.cc.u32 %1, x1, b0, %1;\n\t"
      "madc.lo.cc.u32 %2, x1, b1, %2;\n\t"
      "madc.lo.cc.u32 %3, x1, b2, %3;\n\t"
      "madc.lo.cc.u32 %4, x1, b3, %4;\n\t"
      "addc.u32 %5, %5, 0;\n\t"
      "mad.hi.cc.u32 %2, x1, b0, %2;\n\t"
      "madc.hi.cc.u32 %3, x1, b1, %3;\n\t"
      "madc.hi.cc.u32 %4, x1, b2, %4;\n\t"
      "madc.hi.u32 %5, x1, b3, %5;\n\t"
      "}"
      : "+r"(w[0]), "+r"(w[1]), "+r"(w[2]), "+r"(w[3]), "+r"(w[4]), "+r"(w[5])
      : "l"(x), "l"(blo), "l"(bhi));
}

// w[0..8) (256 bits, 32-bit words) += x * (bhi:blo) for x < 2^64, b < 2^128,
// wrapping modulo 2^256.
__device__ __forceinline__ void mac256(uint32_t* w, uint64_t x, uint64_t blo, uint64_t bhi) {
  asm("{\n\t"
      ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
      "mov.b64 {x0, x1}, %8;\n\t"
      "mov.b64 {b0, b1}, %9;\n\t"
      "mov.b64 {b2, b3}, %10;\n\t"
      "mad.lo.cc.u32 %0, x0, b0, %0;\n\t"
      "madc.lo.cc.u32 %1, x0, b1, %1;\n\t"
      "madc.lo.cc.u32 %2, x0, b2, %2;\n\t"
      "madc.lo.cc.u32 %3, x0, b3, %3;\n\t"
      "addc.cc.u32 %4, %4, 0;\n\t"
      "addc.cc.u32 %5, %5, 0;\n\t"
      "addc.cc.u32 %6, %6, 0;\n\t"
      "addc.u32 %7, %7, 0;\n\t"
      "mad.hi.cc.u32 %1, x0, b0, %1;\n\t"
      "madc.hi.cc.u32 %2, x0, b1, %2;\n\t"
      "madc.hi.cc.u32 %3, x0, b2, %3;\n\t"
      "madc.hi.cc.u32 %4, x0, b3, %4;\n\t"
      "addc.cc.u32 %5, %5, 0;\n\t"
      "addc.cc.u32 %6, %6, 0;\n\t"
      "addc.u32 %7, %7, 0;\n\t"
      "mad.lo.cc.u32 %1, x1, b0, %1;\n\t"
      "madc.lo.cc.u32 %2, x1, b1, %2;\n\t"
      "madc.lo.cc.u32 %3, x1, b2, %3;\n\t"
      "madc.lo.cc.u32 %4, x1, b3, %4;\n\t"
      "addc.cc.u32 %5, %5, 0;\n\t"
      "addc.cc.u32 %6, %6, 0;\n\t"
      "addc.u32 %7, %7, 0;\n\t"
      "mad.hi.cc.u32 %2, x1, b0, %2;\n\t"
      "madc.hi.cc.u32 %3, x1, b1, %3;\n\t"
      "madc.hi.cc.u32 %4, x1, b2, %4;\n\t"
      "madc.hi.cc.u32 %5, x1, b3, %5;\n\t"
      "addc.cc.u32 %6, %6, 0;\n\t"
      "addc.u32 %7, %7, 0;\n\t"
      "}"
      : "+r"(w[0]), "+r"(w[1]), "+r"(w[2]), "+r"(w[3]), "+r"(w[4]), "+r"(w[5]), "+r"(w[6]), "+r"(w[7])
      : "l"(x), "l"(blo), "l"(bhi));
}

// x >= m ? x - m : x with a predicated subtraction.
__device__ __forceinline__ uint64_t csub(uint64_t x, uint64_t m) {
  asm("{\n\t.reg .pred q;\n\tsetp.ge.u64 q, %0, %1;\n\t@q sub.u64 %0, %0, %1;\n\t}" : "+l"(x) : "l"(m));
  return x;
}

__device__ __forceinline__ uint64_t reduce_once(uint64_t x, uint64_t p) { return csub(x, p); }

// (hi * 2^64 + lo) * 2^-64 mod p, canonical, for hi < 4p: hi reduced by two
// conditional subtractions, lo by one Montgomery step (lo * 2^-64 mod p in
// [0, p], as in mont_reduce).
__device__ __forceinline__ uint64_t mont_fold(uint64_t hi, uint64_t lo, uint64_t p, uint64_t pinv) {
  const uint64_t h = csub(csub(hi, 2 * p), p);
  const uint64_t m = lo * pinv;
  return csub(h + __umul64hi(m, p) + (lo != 0), p);
}

__device__ __forceinline__ uint64_t mul_shoup(uint64_t a, uint64_t b, uint64_t b_shoup, uint64_t p) {
  return reduce_once(mul_shoup_lazy(a, b, b_shoup, p), p);
}

// Barrett reduction of the 128-bit value hi:lo into [0, 2p) for hi < 2^63
// (zq/mod.rs:693-707 `lazy_reduce_u128`).
__device__ __forceinline__ uint64_t reduce128_lazy(uint64_t hi, uint64_t lo, const DevPrime& pr) {
  uint64_t t0 = __umul64hi(lo, pr.blo);
  // mid = lo * bhi + hi * blo + t0 (a 129-bit sum kept as hi word + carry)
  uint64_t m1_lo = lo * pr.bhi, m1_hi = __umul64hi(lo, pr.bhi);
  uint64_t m2_lo = hi * pr.blo, m2_hi = __umul64hi(hi, pr.blo);
  uint64_t s = m1_lo + m2_lo;
  uint64_t c = s < m1_lo;
  uint64_t s2 = s + t0;
  c += s2 < s;
  uint64_t q = m1_hi + m2_hi + c + hi * pr.bhi;
  return lo - q * pr.p;
}

__device__ __forceinline__ uint64_t reduce128(uint64_t hi, uint64_t lo, const DevPrime& pr) {
  return reduce_once(reduce128_lazy(hi, lo, pr), pr.p);
}

// a * b mod p for a, b < 2^64 with a * b < 2^126 (Barrett).
__device__ __forceinline__ uint64_t mul_mod(uint64_t a, uint64_t b, const DevPrime& pr) {
  return reduce128(__umul64hi(a, b), a * b, pr);
}

// Asynchronous 16-byte copy global -> shared (no register round trip); the
// copies of a thread complete at cp_async_wait_all (a hardware wait, no
// spinning).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Montgomery reduction of the 128-bit value hi:lo < p * 2^64: returns
// hi:lo * 2^-64 mod p in [0, 2p). With m = lo * (-p^-1) mod 2^64 the sum
// hi:lo + m * p is a multiple of 2^64 whose low word carries exactly when
// lo != 0.
__device__ __forceinline__ uint64_t mont_reduce(uint64_t hi, uint64_t lo, const DevPrime& pr) {
  const uint64_t m = lo * pr.pinv;
  return hi + __umul64hi(m, pr.p) + (lo != 0);
}

// Lazy reduction of a single word into [0, 2p) (zq/mod.rs:712-723 `lazy_reduce`).
__device__ __forceinline__ uint64_t reduce64_lazy(uint64_t a, const DevPrime& pr) {
  // q = floor((a * bhi + floor(a * blo / 2^64)) / 2^64)
  uint64_t t = __umul64hi(a, pr.blo);
  uint64_t lo = a * pr.bhi;
  uint64_t hi = __umul64hi(a, pr.bhi);
  uint64_t s = lo + t;
  hi += s < lo;
  return a - hi * pr.p;
}

__device__ __forceinline__ uint64_t add_mod(uint64_t a, uint64_t b, uint64_t p) { return reduce_once(a + b, p); }
__device__ __forceinline__ uint64_t sub_mod(uint64_t a, uint64_t b, uint64_t p) { return reduce_once(a + p - b, p); }

// Harvey forward butterfly (native.rs:256-269): x, y in [0, 4p) -> [0, 4p).
__device__ __forceinline__ void fwd_bfly(uint64_t& x, uint64_t& y, uint64_t w, uint64_t ws, uint64_t p,
                                         uint64_t p2) {
  const uint64_t a = csub(x, p2);
  const uint64_t t = mul_shoup_lazy(y, w, ws, p);
  x = a + t;
  y = a + p2 - t;
}

// Gentleman-Sande inverse butterfly (native.rs:288-300): x, y in [0, 2p).
__device__ __forceinline__ void inv_bfly(uint64_t& x, uint64_t& y, uint64_t z, uint64_t zs, uint64_t p,
                                         uint64_t p2) {
  const uint64_t t = x;
  x = csub(x + y, p2);
  y = mul_shoup_lazy(t + p2 - y, z, zs, p);
}

// The last Gentleman-Sande stage followed by the final scale s (N^-1 or its
// Montgomery form), with zs = z * s precomputed: x, y in [0, 2p) become the
// canonical ((x + y) s, (x - y) z s) mod p, the values the reference's
// butterfly and scaling produce, with two products instead of three.
__device__ __forceinline__ void inv_bfly_final(uint64_t& x, uint64_t& y, uint64_t zs, uint64_t zs_shoup, uint64_t s,
                                               uint64_t s_shoup, uint64_t p, uint64_t p2) {
  const uint64_t t = x;
  x = mul_shoup(x + y, s, s_shoup, p);
  y = mul_shoup(t + p2 - y, zs, zs_shoup, p);
}

// native.rs:238-243 `reduce3`: [0, 4p) -> [0, p).
__device__ __forceinline__ uint64_t reduce4(uint64_t x, uint64_t p, uint64_t p2) { return csub(csub(x, p2), p); }

}  // namespace fheg
