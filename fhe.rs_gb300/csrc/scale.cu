// RNS scaling (fhe-math `rns/scaler.rs`, `rq/scaler.rs`): the CUDA-core
// kernels and, for the exact source counts, the tensor-core form (byte-sliced
// products on tcgen05).

#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_fp16.h>

#include "lib.hpp"
#include "ntt.cuh"
#include "tc.cuh"

namespace fheg {

static unsigned blocks_for(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }
// ---------------------------------------------------------------------------
// RNS scaling (rns/scaler.rs:249-352), one thread per coefficient.
//
// The reference accumulates in wrapping 256-bit integers; the sums here are
// the same integers accumulated exactly in 32-bit words:
//   G = sum_k r_k * theta_garner_k           (< 2^192 by the choice of shift)
//   O = sum_k (+/-) r_k * theta_omega_k - (+/-) v * theta_gamma   (mod 2^256)
// and each output residue is one exact dot product reduced once:
//   y_j = sum_k r_k * omega_jk + v_j * (q_j - gamma_j) + w_term  (mod q_j),
// which equals the reference's lazily reduced sum modulo q_j.

__device__ __forceinline__ uint64_t join(uint32_t lo, uint32_t hi) { return ((uint64_t)hi << 32) | lo; }

// Low 128 bits of (w >> s) for an nw-word little-endian value (32-bit words).
__device__ __forceinline__ void shr_words(const uint32_t* w, int nw, uint32_t s, uint64_t* lo, uint64_t* hi) {
  uint32_t o[4];
  const uint32_t ws = s >> 5, bs = s & 31;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const uint32_t idx = ws + k;
    uint32_t a = 0, b = 0;
#pragma unroll
    for (int m = 0; m < 8; m++) {
      if (m < nw && (uint32_t)m == idx) a = w[m];
      if (m < nw && (uint32_t)m == idx + 1) b = w[m];
    }
    o[k] = bs ? ((a >> bs) | (b << (32 - bs))) : a;
  }
  *lo = join(o[0], o[1]);
  *hi = join(o[2], o[3]);
}

// 256-bit a += b, a -= b (32-bit words).
__device__ __forceinline__ void add256w(uint32_t* a, const uint32_t* b) {
  asm("add.cc.u32 %0, %0, %8;\n\taddc.cc.u32 %1, %1, %9;\n\taddc.cc.u32 %2, %2, %10;\n\taddc.cc.u32 %3, %3, %11;\n\t"
      "addc.cc.u32 %4, %4, %12;\n\taddc.cc.u32 %5, %5, %13;\n\taddc.cc.u32 %6, %6, %14;\n\taddc.u32 %7, %7, %15;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void sub256w(uint32_t* a, const uint32_t* b) {
  asm("sub.cc.u32 %0, %0, %8;\n\tsubc.cc.u32 %1, %1, %9;\n\tsubc.cc.u32 %2, %2, %10;\n\tsubc.cc.u32 %3, %3, %11;\n\t"
      "subc.cc.u32 %4, %4, %12;\n\tsubc.cc.u32 %5, %5, %13;\n\tsubc.cc.u32 %6, %6, %14;\n\tsubc.u32 %7, %7, %15;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4]), "+r"(a[5]), "+r"(a[6]), "+r"(a[7])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

// High parts of the scaler's sums. The sums only matter at bit 96 and above
// (v needs G >> (shift - 1) with shift >= 123, w needs S >> 126), so the
// fast path adds only the partial products x_i b_j (32-bit words) that
// reach word 3: those with i + j >= 3, and the high halves of those with
// i + j = 2. The rest of a term x * b (x < 2^64, b < 2^128) is below
// 2^64 + 4 * 2^96 < 5 * 2^96, so a sum of F such terms is its kept part (a
// multiple of 2^96) plus less than 5F * 2^96; a result whose kept part is
// that close to a rounding boundary is recomputed exactly.
//
// h[0..NH) are words 3 .. 2 + NH of the sum: NH = 3 for a sum below 2^192,
// NH = 5 for a sum taken modulo 2^256.
template <int NH>
__device__ __forceinline__ void mac_hi(uint32_t* h, uint64_t x, uint64_t blo, uint64_t bhi) {
  static_assert(NH == 3 || NH == 5, "three or five high words");
  if constexpr (NH == 3) {
    asm("{\n\t"
        ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
        "mov.b64 {x0, x1}, %3;\n\t"
        "mov.b64 {b0, b1}, %4;\n\t"
        "mov.b64 {b2, b3}, %5;\n\t"
        "mad.hi.cc.u32 %0, x0, b2, %0;\n\t"
        "madc.hi.cc.u32 %1, x0, b3, %1;\n\t"
        "madc.hi.u32 %2, x1, b3, %2;\n\t"
        "mad.lo.cc.u32 %0, x0, b3, %0;\n\t"
        "madc.lo.cc.u32 %1, x1, b3, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "mad.hi.cc.u32 %0, x1, b1, %0;\n\t"
        "madc.hi.cc.u32 %1, x1, b2, %1;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "mad.lo.cc.u32 %0, x1, b2, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.u32 %2, %2, 0;\n\t"
        "}"
        : "+r"(h[0]), "+r"(h[1]), "+r"(h[2])
        : "l"(x), "l"(blo), "l"(bhi));
  } else {
    asm("{\n\t"
        ".reg .u32 x0, x1, b0, b1, b2, b3;\n\t"
        "mov.b64 {x0, x1}, %5;\n\t"
        "mov.b64 {b0, b1}, %6;\n\t"
        "mov.b64 {b2, b3}, %7;\n\t"
        "mad.hi.cc.u32 %0, x0, b2, %0;\n\t"
        "madc.hi.cc.u32 %1, x0, b3, %1;\n\t"
        "madc.hi.cc.u32 %2, x1, b3, %2;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %0, x0, b3, %0;\n\t"
        "madc.lo.cc.u32 %1, x1, b3, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.hi.cc.u32 %0, x1, b1, %0;\n\t"
        "madc.hi.cc.u32 %1, x1, b2, %1;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "mad.lo.cc.u32 %0, x1, b2, %0;\n\t"
        "addc.cc.u32 %1, %1, 0;\n\t"
        "addc.cc.u32 %2, %2, 0;\n\t"
        "addc.cc.u32 %3, %3, 0;\n\t"
        "addc.u32 %4, %4, 0;\n\t"
        "}"
        : "+r"(h[0]), "+r"(h[1]), "+r"(h[2]), "+r"(h[3]), "+r"(h[4])
        : "l"(x), "l"(blo), "l"(bhi));
  }
}

// Words 3..7 of v * theta_gamma for v < 2^96 (vlo, vhi, vhi < 2^32), kept
// as in mac_hi: the low 64 bits of v through mac_hi (dropping less than
// 5 * 2^96), the third word's partial products at word 2 and above (dropping
// the low half of its lowest one, less than 2^96).
__device__ __forceinline__ void mul_v_hi(uint32_t* h, uint64_t vlo, uint64_t vhi, uint64_t blo, uint64_t bhi) {
#pragma unroll
  for (int k = 0; k < 5; k++) h[k] = 0;
  mac_hi<5>(h, vlo, blo, bhi);
  asm("{\n\t"
      ".reg .u32 v2, b0, b1, b2, b3;\n\t"
      "cvt.u32.u64 v2, %5;\n\t"
      "mov.b64 {b0, b1}, %6;\n\t"
      "mov.b64 {b2, b3}, %7;\n\t"
      "mad.hi.cc.u32 %0, v2, b0, %0;\n\t"
      "madc.hi.cc.u32 %1, v2, b1, %1;\n\t"
      "madc.hi.cc.u32 %2, v2, b2, %2;\n\t"
      "madc.hi.cc.u32 %3, v2, b3, %3;\n\t"
      "addc.u32 %4, %4, 0;\n\t"
      "mad.lo.cc.u32 %0, v2, b1, %0;\n\t"
      "madc.lo.cc.u32 %1, v2, b2, %1;\n\t"
      "madc.lo.cc.u32 %2, v2, b3, %2;\n\t"
      "addc.cc.u32 %3, %3, 0;\n\t"
      "addc.u32 %4, %4, 0;\n\t"
      "}"
      : "+r"(h[0]), "+r"(h[1]), "+r"(h[2]), "+r"(h[3]), "+r"(h[4])
      : "l"(vhi), "l"(blo), "l"(bhi));
}

// 160-bit a += b, a -= b (32-bit words).
__device__ __forceinline__ void add160w(uint32_t* a, const uint32_t* b) {
  asm("add.cc.u32 %0, %0, %5;\n\taddc.cc.u32 %1, %1, %6;\n\taddc.cc.u32 %2, %2, %7;\n\taddc.cc.u32 %3, %3, %8;\n\t"
      "addc.u32 %4, %4, %9;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]));
}

__device__ __forceinline__ void sub160w(uint32_t* a, const uint32_t* b) {
  asm("sub.cc.u32 %0, %0, %5;\n\tsubc.cc.u32 %1, %1, %6;\n\tsubc.cc.u32 %2, %2, %7;\n\tsubc.cc.u32 %3, %3, %8;\n\t"
      "subc.u32 %4, %4, %9;"
      : "+r"(a[0]), "+r"(a[1]), "+r"(a[2]), "+r"(a[3]), "+r"(a[4])
      : "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]));
}

// Full 128 x 128 -> 256-bit product (32-bit words).
__device__ __forceinline__ void mul128x128w(uint32_t* r, uint64_t alo, uint64_t ahi, uint64_t blo, uint64_t bhi) {
#pragma unroll
  for (int k = 0; k < 8; k++) r[k] = 0;
  uint32_t t[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  mac256(t, alo, blo, bhi);  // alo * b at word 0
  uint32_t hi6[6] = {0, 0, 0, 0, 0, 0};
  mac192(hi6, ahi, blo, bhi);  // ahi * b at word 2 (< 2^192)
  uint32_t u[8] = {0, 0, hi6[0], hi6[1], hi6[2], hi6[3], hi6[4], hi6[5]};
  add256w(t, u);
#pragma unroll
  for (int k = 0; k < 8; k++) r[k] = t[k];
}

// All constants of one launch travel in the kernel's parameter space, so
// every multiply-add reads its constant operand straight from the constant
// bank (fully unrolled loops give compile-time offsets). Outputs are limbs
// start .. start + out_len of the target; the rows of omega, gamma and the
// primes are pre-sliced on the host so output o uses row o.
//
// Kernels with an exact source count (EXACT) take odd target moduli, with
// omega, gamma_neg and gamma_neg_hi in Montgomery form (times 2^64 mod q_j):
// the exact sum S is then 2^64 times the output's sum, and one Montgomery
// step divides it back out (mont_fold), with about a third of the multiplies
// of a 128-bit Barrett reduction. The generic kernels take plain constants
// and reduce S by Barrett (any moduli).
template <int MAXF, int MAXT>
struct RnsLaunch {
  uint32_t from_len, out_len, is_one, shift;
  uint32_t tg_sign, to_sign;  // to_sign: bit k = sign of theta_omega_k
  uint64_t tg_lo, tg_hi;
  uint64_t tgar_lo[MAXF], tgar_hi[MAXF];
  uint64_t to_lo[MAXF], to_hi[MAXF];
  uint64_t omega[MAXT][MAXF];
  uint64_t gamma_neg[MAXT];     // (q_j - gamma_j) mod q_j
  uint64_t gamma_neg_hi[MAXT];  // gamma_neg * 2^62 mod q_j
  uint64_t p[MAXT], bhi[MAXT], blo[MAXT];
  uint64_t pinv[MAXT];  // -q_j^-1 mod 2^64 (EXACT)
  // w mod q_j as whi * (2^64 mod q_j) + wlo (EXACT): the Shoup companions of
  // 2^64 mod q_j and of 1, and wbig = every q_j above 2^61 (wlo < 8 q_j).
  uint32_t wbig;
  uint64_t r64[MAXT], r64_shoup[MAXT], one_shoup[MAXT];
};


// EXACT: the source count is MAXF itself (a compile-time constant), so the
// unrolled loops carry no predicated-off terms; used for the counts the
// default multiplications produce (L and 2L + 1 source moduli).
//
// TOP > 0: `in` holds the block pass of a two-pass inverse NTT whose last TOP
// strided stages and final scale have not run. Each CTA of 128 threads then
// owns the 128 coefficients b + t * 2^(logn - TOP) of 128 >> TOP groups b
// (t < 2^TOP); it applies those stages to every source limb of its groups
// (inv_top_stages, the strided inverse pass's arithmetic) into shared memory,
// and each thread scales one coefficient from there. The strided pass and
// its round trip through HBM disappear; the results are the same.
//
// With TOP > 0 and fwd_primes set, the outputs are themselves the input of a
// two-pass forward NTT whose strided first TOP stages this kernel applies
// (fwd_top_stages, output limb o in fwd_primes[o]): they go through shared
// memory so that each group's 2^TOP coefficients meet, and leave lazy in
// [0, 4p) for the block pass.
template <int WORDS>
__device__ __forceinline__ uint64_t* rns_stage_buffer() {
  __shared__ uint64_t buf[WORDS];
  return buf;
}

// Forward stages of the kernel's epilogue (ForwardTop for one launch; primes
// null: none).
struct FwdEpilogue {
  const DevPrime* primes;
  uint32_t period, take;
  const DevPrime* digit_primes;
  uint32_t digit_limbs, digit_raw;
  PolyRef digits;
};

// The exact sums of the rare coefficients whose fast high-word sums sit next
// to a rounding boundary, kept out of line so that the hot kernel body stays
// small in the instruction cache: G (six words) and S (eight words, mod
// 2^256) as the reference accumulates them.
template <int MAXF, int MAXT>
__device__ __noinline__ void rns_exact_g(const RnsLaunch<MAXF, MAXT>* s, const uint64_t* r, uint32_t F, uint32_t* g) {
#pragma unroll 1
  for (int k = 0; k < 6; k++) g[k] = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < F; k++) mac192(g, r[k], s->tgar_lo[k], s->tgar_hi[k]);
}

template <int MAXF, int MAXT>
__device__ __noinline__ void rns_exact_s(const RnsLaunch<MAXF, MAXT>* s, const uint64_t* r, uint32_t F, uint64_t vlo,
                                        uint64_t vhi, uint32_t* pos) {
  uint32_t neg[8];
#pragma unroll 1
  for (int k = 0; k < 8; k++) pos[k] = neg[k] = 0;
#pragma unroll 1
  for (uint32_t k = 0; k < F; k++) {
    if ((s->to_sign >> k) & 1) mac256(neg, r[k], s->to_lo[k], s->to_hi[k]);
    else mac256(pos, r[k], s->to_lo[k], s->to_hi[k]);
  }
  sub256w(pos, neg);
  uint32_t vt[8];
  mul128x128w(vt, vlo, vhi, s->tg_lo, s->tg_hi);
  if (s->tg_sign) add256w(pos, vt);
  else sub256w(pos, vt);
}

// The tensor-core form (TC) of the exact kernels. Every sum the scaler forms
// is a product of the source residues r_k with constants X_k: G (theta_garner,
// exact), S (+/- theta_omega, mod 2^256) and each output's sum (omega_jk times
// 2^64 mod q_j). Writing r_k = sum_b a_kb 2^(8b) with bytes a_kb, and the
// constants X_kb = X_k 2^(8b) (exact, mod 2^256, mod q_j) in bytes x_kbc,
//   sum_k r_k X_k = sum_c 2^(8c) D_c,  D_c = sum_(k,b) a_kb x_kbc,
// a matrix product of the 128 x 8F byte matrix of a CTA's coefficients with
// the 8F x N byte matrix of the launch. Bytes are exact FP16 values, every
// product is below 2^16 and every D_c below 8F * 2^16 <= 2^24 (F <= 32), so
// tcgen05's FP16 MMA with FP32 accumulation in tensor memory computes the D_c
// exactly (below 2^23 for F <= 16, which lets a float addition turn them into
// integers; above, a conversion instruction does). Each thread then reads its
// row and carries the D_c into the words of G, S and the output sums on the
// CUDA cores, instead of the multiply-adds of the unrolled sums (about 300
// 32-bit ones per coefficient for the L = 6 scale-down).
//
// Column groups of 8 (one group = 8 bytes of one sum): 0-2 G, 3-6 S, then one
// per output modulus. A launch runs two passes through the same tensor-memory
// columns: pass 0 multiplies by the groups of G (and S unless the factor is
// one), pass 1 by the groups of its output slice; each pass's operand B is
// bulk-copied from the scaler's matrix into one shared buffer (pass 1's copy
// once pass 0's MMAs are done with it). N of a pass is 8 groups rounded up to
// a multiple of 16; the rows beyond its groups hold stale bytes whose columns
// are never read.
//
// Split form (a scale-down whose operand buffer would otherwise cost an SM a
// CTA): four passes through a smaller buffer, G into columns 0-31, S into
// 32-63, the first `chunk` outputs into 64.., and once every thread has read
// G and S, the other outputs into 0.. .
struct TcMat {
  const uint16_t* mat;   // FP16 bit patterns, 16 * kp bytes per group (tc.cuh layout)
  uint32_t kp;           // 8 F rounded up to a multiple of 16
  uint32_t head_groups;  // G (and S) groups: 3 or 7
  uint32_t out_group0;   // first output group of the launch (7 + start)
  uint32_t n0, n1;       // N of pass 0 (G and S; split: G) and of the (first) output pass
  uint32_t cols;         // tensor-memory columns allocated (64 or 128)
  uint32_t b_offset;     // byte offset of B in the dynamic shared memory
  uint32_t chunk, n2;    // split form: outputs of the first output pass, N of the second
};

// Count of waits of the tensor-core scaler that ran out (the MMA or the
// operand copy did not complete in time); read by rns_tc_wait_failures.
__device__ uint32_t g_tc_wait_failures;

constexpr uint32_t kTcWaitTries = 1u << 20;

// Thread 0: the MMAs of pass `phase` (K / 16 of them, N = n, into the
// columns at `tmem`) once its operand B has landed (that phase of bar_b),
// committed to bar_mma, the pass's own single-use barrier (waited at parity
// 0: a barrier shared by several passes aliases their phases for a thread
// that waits after two of them have completed). A copy that does not land in
// time is counted, the pass's MMAs are skipped (its outputs are then not
// valid) and bar_mma is released by hand so that no thread waits longer than
// its own bounded wait.
template <uint32_t KP>
__device__ __forceinline__ void tc_pass(uint32_t bar_b, uint32_t bar_mma, uint32_t phase, uint32_t tmem, uint32_t sa,
                                        uint32_t sb, uint32_t n) {
  if (mbar_wait(bar_b, phase & 1, kTcWaitTries)) {
    const uint32_t idesc = tc_idesc_f16_f32(128, n);
#pragma unroll
    for (uint32_t kk = 0; kk < KP / 16; kk++)
      tc_mma_f16(tmem, tc_smem_desc(sa + kk * 256, 16 * KP), tc_smem_desc(sb + kk * 256, 16 * KP), idesc,
                 kk > 0 ? 1u : 0u);
    tc_commit(bar_mma);
  } else {
    atomicAdd(&g_tc_wait_failures, 1u);
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar_mma) : "memory");
    mbar_wait(bar_b, phase & 1, kTcWaitTries);
  }
}

// Two bytes of w (prmt selector sel) as the half2 (b0, b1): 0x64bb is the
// FP16 value 1024 + b, less 1024.
__device__ __forceinline__ uint32_t tc_bytes_half2(uint32_t w, uint32_t sel) {
  uint32_t t;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(t) : "r"(w), "r"(0x64646464u), "r"(sel));
  __half2 h = *reinterpret_cast<__half2*>(&t);
  h = __hsub2(h, __halves2half2(__ushort_as_half(0x6400), __ushort_as_half(0x6400)));
  return *reinterpret_cast<uint32_t*>(&h);
}

// An exact FP32 integer as an integer: below 2^23 (SMALL), its mantissa after
// adding 2^23; below 2^24, by conversion.
template <bool SMALL>
__device__ __forceinline__ uint32_t tc_int(uint32_t f) {
  if constexpr (SMALL) return __float_as_uint(__fadd_rn(__uint_as_float(f), 8388608.0f)) - 0x4B000000u;
  else return __float2uint_rz(__uint_as_float(f));
}

// Carries one group (8 column sums D_c, c = 8q .. 8q + 7, each below 2^24)
// into two 32-bit words of sum_c 2^(8c) D_c; acc holds the carry between
// groups.
template <bool SMALL>
__device__ __forceinline__ void tc_words(const uint32_t* c, uint64_t& acc, uint32_t* w) {
  acc += (uint64_t)tc_int<SMALL>(c[0]) + ((uint64_t)tc_int<SMALL>(c[1]) << 8) +
         ((uint64_t)tc_int<SMALL>(c[2]) << 16) + ((uint64_t)tc_int<SMALL>(c[3]) << 24);
  w[0] = (uint32_t)acc;
  acc >>= 32;
  acc += (uint64_t)tc_int<SMALL>(c[4]) + ((uint64_t)tc_int<SMALL>(c[5]) << 8) +
         ((uint64_t)tc_int<SMALL>(c[6]) << 16) + ((uint64_t)tc_int<SMALL>(c[7]) << 24);
  w[1] = (uint32_t)acc;
  acc >>= 32;
}

// The dynamic shared memory of a TC launch: the stage buffer, overlaid by A
// (128 x KP FP16) once the residues are in registers, then B.
__device__ __forceinline__ uint8_t* tc_dyn_smem() {
  extern __shared__ __align__(128) uint8_t tc_dyn[];
  return tc_dyn;
}

template <int WORDS, bool TC>
__device__ __forceinline__ uint64_t* scale_stage() {
  if constexpr (TC) return reinterpret_cast<uint64_t*>(tc_dyn_smem());
  else return rns_stage_buffer<WORDS>();
}

// FASTV: the kept-high-word sums below, with exact fallbacks. They are exact
// for every scaler; on GB300 they shortened the extension of the L = 6
// multiplication (6 source moduli, factor one) by 4% and lengthened its
// scale-down (13 source moduli, which also forms w) by 15%, so only the
// extensions' source counts use them and the rest sum exactly inline.
//
// TC (EXACT, 12 <= F <= 32): the sums come from the tensor core (above); every
// CTA covers 128 coefficients with all its threads and holds 64 or 128
// tensor-memory columns and at least 456 bytes of shared memory per column,
// so that the CTAs an SM holds never ask for more than its 512 columns. The
// stage buffer then lives in the dynamic shared memory, where A overlays it
// once every thread holds its residues. SPLIT (with TC): the split form, a
// kernel of its own so that the two-pass form carries none of its branches.
template <int MAXF, int MAXT, bool EXACT, int TOP, bool FASTV, bool TC, bool SPLIT = false>
__global__ void __launch_bounds__(128) k_rns_scale(const __grid_constant__ RnsLaunch<MAXF, MAXT> s, uint32_t logn,
                                                   PolyRef in, PolyRef out, uint64_t total,
                                                   const DevPrime* src_primes, uint32_t src_mont,
                                                   const FwdEpilogue fe, const TcMat tc) {
  const uint32_t F = EXACT ? (uint32_t)MAXF : s.from_len;
  constexpr int G = 128 >> TOP;  // groups per CTA (TOP > 0)
  constexpr uint32_t KP = (8 * MAXF + 15) / 16 * 16;
  uint32_t i, poly, b0 = 0, logb = 0, t = 0, gi = 0;
  bool fwd_here = false, dig_here = false;  // uniform across the CTA (one polynomial)
  uint64_t r[MAXF];
  [[maybe_unused]] uint32_t tmem = 0, bar_b = 0, bar_mma = 0;  // bar_mma: pass 0's; pass p's is bar_mma + 8 p
  [[maybe_unused]] uint8_t* tc_a = nullptr;
  [[maybe_unused]] __shared__ __align__(8) uint64_t tc_bars[TC ? 5 : 1];
  [[maybe_unused]] __shared__ uint32_t tc_slot;
  if constexpr (TC) {
    // Operand B in flight and the tensor memory allocated while the sources
    // load.
    tc_a = tc_dyn_smem();
    uint8_t* tc_b = tc_a + tc.b_offset;
    bar_b = smem_u32(&tc_bars[0]);
    bar_mma = smem_u32(&tc_bars[1]);
    const uint32_t group_bytes = 16 * KP;
    if (threadIdx.x == 0) {
      mbar_init(bar_b, 1);
#pragma unroll
      for (uint32_t p = 0; p < 4; p++) mbar_init(bar_mma + 8 * p, 1);
      fence_proxy_async_smem();
      const uint32_t first = (SPLIT ? 3 : tc.head_groups) * group_bytes;
      mbar_expect_tx(bar_b, first);
      bulk_g2s(smem_u32(tc_b), tc.mat, first, bar_b);
    }
    if ((threadIdx.x >> 5) == 1) tc_alloc(smem_u32(&tc_slot), tc.cols);
  }
  if constexpr (TOP == 0) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    i = gid & ((1u << logn) - 1);
    poly = (uint32_t)(gid >> logn);
    const uint64_t* src = in.at(poly, 0) + i;
#pragma unroll
    for (int k = 0; k < MAXF; k++) r[k] = k < (int)F ? src[(uint64_t)k << logn] : 0;
  } else {
    // The grid covers whole polynomials (2^logn is a multiple of 128), so
    // every thread reaches the barriers.
    uint64_t* staged = scale_stage<(MAXF > MAXT ? MAXF : MAXT) * 128, TC>();
    poly = blockIdx.x >> (logn - 7);
    b0 = (blockIdx.x & ((1u << (logn - 7)) - 1)) * G;
    logb = logn - TOP;
    if constexpr (TC) {
      // Every load of the thread's items issued before the first use (the
      // tensor-core form runs fewer warps per SM; the CUDA-core kernels,
      // with more warps and fewer registers, measured faster without).
      constexpr int IT = (MAXF * G + 127) / 128;
      uint64_t x[IT][1 << TOP];
#pragma unroll
      for (int u = 0; u < IT; u++) {
        const uint32_t item = threadIdx.x + 128 * u;
        if (item < F * G) {
          const uint64_t* row = in.at(poly, item / G) + b0 + item % G;
#pragma unroll
          for (int t = 0; t < (1 << TOP); t++) x[u][t] = row[(uint64_t)t << logb];
        }
      }
#pragma unroll
      for (int u = 0; u < IT; u++) {
        const uint32_t item = threadIdx.x + 128 * u;
        if (item < F * G) {
          const uint32_t k = item / G, gi = item % G;
          inv_top_stages<TOP>(x[u], src_primes[k], 1u << logn, src_mont != 0);
#pragma unroll
          for (int t = 0; t < (1 << TOP); t++) staged[(k * (1 << TOP) + t) * G + gi] = x[u][t];
        }
      }
    } else {
      for (uint32_t item = threadIdx.x; item < F * G; item += 128) {
        const uint32_t k = item / G, gi = item % G;
        const uint64_t* row = in.at(poly, k) + b0 + gi;
        uint64_t x[1 << TOP];
#pragma unroll
        for (int t = 0; t < (1 << TOP); t++) x[t] = row[(uint64_t)t << logb];
        inv_top_stages<TOP>(x, src_primes[k], 1u << logn, src_mont != 0);
#pragma unroll
        for (int t = 0; t < (1 << TOP); t++) staged[(k * (1 << TOP) + t) * G + gi] = x[t];
      }
    }
    __syncthreads();
    t = threadIdx.x / G;
    gi = threadIdx.x % G;
    i = b0 + gi + (t << logb);
#pragma unroll
    for (int k = 0; k < MAXF; k++) r[k] = k < (int)F ? staged[(k * (1 << TOP) + t) * G + gi] : 0;
    if (fe.primes) {
      const uint32_t part = fe.period ? poly % fe.period : 0;
      fwd_here = part < fe.take;
      dig_here = !fwd_here && fe.digit_primes != nullptr;
    }
    // The buffer takes the outputs next (TC: A first).
    if (TC || fwd_here || dig_here) __syncthreads();
  }

  [[maybe_unused]] uint32_t lane = 0;
  if constexpr (TC) {
    // Row threadIdx.x of A: the bytes of the thread's residues, one 16-byte
    // core-matrix row per residue, zeros beyond F.
#pragma unroll
    for (uint32_t l = 0; l < KP / 8; l++) {
      uint4 v = make_uint4(0, 0, 0, 0);
      if (l < F) {
        const uint32_t lo = (uint32_t)r[l], hi = (uint32_t)(r[l] >> 32);
        v = make_uint4(tc_bytes_half2(lo, 0x4140), tc_bytes_half2(lo, 0x4342), tc_bytes_half2(hi, 0x4140),
                       tc_bytes_half2(hi, 0x4342));
      }
      *reinterpret_cast<uint4*>(tc_a + tc_core_off(threadIdx.x, 8 * l, KP)) = v;
    }
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tmem = tc_slot;
    const uint32_t sa = smem_u32(tc_a), sb = sa + tc.b_offset;
    if (threadIdx.x == 0) tc_pass<KP>(bar_b, bar_mma, 0, tmem, sa, sb, tc.n0);
    if (!mbar_wait(bar_mma, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
    tc_fence_after();
    // Pass 0's MMAs are done with B: pass 1's operand (S when split, else the
    // outputs) lands while its columns are read.
    if (threadIdx.x == 0) {
      const uint32_t group_bytes = 16 * KP;
      const uint32_t g0 = SPLIT ? 3 : tc.out_group0, ng = SPLIT ? 4 : s.out_len;
      mbar_expect_tx(bar_b, ng * group_bytes);
      bulk_g2s(sb, reinterpret_cast<const uint8_t*>(tc.mat) + g0 * group_bytes, ng * group_bytes, bar_b);
    }
    lane = tmem + (((threadIdx.x >> 5) * 32u) << 16);
  }

  // scaler.rs:260-272: v = ceil((G >> (shift - 1)) / 2). Fast path (FASTV): the
  // kept high words of G; exact when G >> (shift - 1) cannot change under
  // the dropped part (below 5F * 2^96): (H mod 2^e) + 5F < 2^e, e = shift - 97.
  uint32_t g[6] = {0, 0, 0, 0, 0, 0};
  bool exact = true;
  // TC: the column sums of G (24) and S (32) in one tensor-memory round trip.
  [[maybe_unused]] uint32_t gs[TC ? 56 : 1];
  if constexpr (TC) {
    const uint32_t sa = smem_u32(tc_a), sb = sa + tc.b_offset;
    if constexpr (!SPLIT) {
      if (s.is_one) tc_ld24(lane, gs);
      else tc_ld56(lane, gs);
      // Every lane's pass-0 columns are read: pass 1 may overwrite them, and
      // its MMAs run while the sums below are carried and rounded.
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (threadIdx.x == 0) tc_pass<KP>(bar_b, bar_mma + 8, 1, tmem, sa, sb, tc.n1);
    } else {
      // S (pass 1) into columns 32-63 while G is read.
      if (threadIdx.x == 0) tc_pass<KP>(bar_b, bar_mma + 8, 1, tmem + 32, sa, sb, 32);
      tc_ld24(lane, gs);
      if (!mbar_wait(bar_mma + 8, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
      tc_fence_after();
      const uint32_t group_bytes = 16 * KP;
      if (threadIdx.x == 0) {
        mbar_expect_tx(bar_b, tc.chunk * group_bytes);
        bulk_g2s(sb, reinterpret_cast<const uint8_t*>(tc.mat) + tc.out_group0 * group_bytes, tc.chunk * group_bytes,
                 bar_b);
      }
      tc_ld32(lane + 32, gs + 24);
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      // The first outputs (pass 2) into columns 64.., then, once their MMAs
      // are done with B, the others (pass 3) over G and S.
      if (threadIdx.x == 0) {
        tc_pass<KP>(bar_b, bar_mma + 16, 2, tmem + 64, sa, sb, tc.n1);
        if (!mbar_wait(bar_mma + 16, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
        tc_fence_after();
        const uint32_t rest = s.out_len - tc.chunk;
        mbar_expect_tx(bar_b, rest * group_bytes);
        bulk_g2s(sb, reinterpret_cast<const uint8_t*>(tc.mat) + (tc.out_group0 + tc.chunk) * group_bytes,
                 rest * group_bytes, bar_b);
        tc_pass<KP>(bar_b, bar_mma + 24, 3, tmem, sa, sb, tc.n2);
      }
    }
    uint64_t acc = 0;
#pragma unroll
    for (uint32_t q = 0; q < 3; q++) tc_words<(MAXF <= 16)>(gs + 8 * q, acc, g + 2 * q);
  } else if constexpr (FASTV) {
#pragma unroll
    for (int k = 0; k < MAXF; k++)
      if (k < (int)F) mac_hi<3>(g + 3, r[k], s.tgar_lo[k], s.tgar_hi[k]);
    // shift >= 122 for any source count up to 128 moduli below 2^62; smaller
    // shifts (never produced) take the exact path.
    const uint32_t e_bits = s.shift >= 104 ? s.shift - 97 : 7;
    exact = s.shift < 104 || (g[3] & ((1u << e_bits) - 1)) >= (1u << e_bits) - 5 * F;
    if (exact) rns_exact_g<MAXF, MAXT>(&s, r, F, g);
  } else {
#pragma unroll
    for (int k = 0; k < MAXF; k++)
      if (k < (int)F) mac192(g, r[k], s.tgar_lo[k], s.tgar_hi[k]);
  }
  uint64_t vlo, vhi;
  shr_words(g, 6, s.shift - 1, &vlo, &vhi);
  {
    const uint64_t odd = vlo & 1;
    vlo = (vlo >> 1) | (vhi << 63);
    vhi >>= 1;
    vlo += odd;
    vhi += (vlo < odd);
  }

  // scaler.rs:276-314. Fast path (FASTV): the kept high words of the signed sum S
  // (the dropped part lies in (-(5F + 6), 5F + 6) * 2^96: 5 * 2^96 per term
  // and 6 * 2^96 for v * theta_gamma); exact when S >> 126 cannot change,
  // i.e. H mod 2^30 is at least 5F + 6 away from a multiple of 2^30.
  bool w_sign = false;
  uint64_t wlo = 0, whi = 0;
  if (!s.is_one) {
    uint32_t pos[8] = {0, 0, 0, 0, 0, 0, 0, 0}, neg[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if constexpr (TC) {
      uint64_t acc = 0;
#pragma unroll
      for (uint32_t q = 0; q < 4; q++) tc_words<(MAXF <= 16)>(gs + 24 + 8 * q, acc, pos + 2 * q);
      uint32_t vt[8];
      mul128x128w(vt, vlo, vhi, s.tg_lo, s.tg_hi);
      if (s.tg_sign) add256w(pos, vt);
      else sub256w(pos, vt);
      exact = false;
    } else if constexpr (!FASTV) {
#pragma unroll
      for (int k = 0; k < MAXF; k++) {
        if (k < (int)F) {
          if ((s.to_sign >> k) & 1) mac256(neg, r[k], s.to_lo[k], s.to_hi[k]);
          else mac256(pos, r[k], s.to_lo[k], s.to_hi[k]);
        }
      }
      sub256w(pos, neg);
      uint32_t vt[8];
      mul128x128w(vt, vlo, vhi, s.tg_lo, s.tg_hi);
      if (s.tg_sign) add256w(pos, vt);
      else sub256w(pos, vt);
      exact = false;
    } else if (!exact) {
#pragma unroll
      for (int k = 0; k < MAXF; k++) {
        if (k < (int)F) {
          if ((s.to_sign >> k) & 1) mac_hi<5>(neg + 3, r[k], s.to_lo[k], s.to_hi[k]);
          else mac_hi<5>(pos + 3, r[k], s.to_lo[k], s.to_hi[k]);
        }
      }
      sub160w(pos + 3, neg + 3);
      uint32_t vt[5];
      mul_v_hi(vt, vlo, vhi, s.tg_lo, s.tg_hi);
      if (s.tg_sign) add160w(pos + 3, vt);
      else sub160w(pos + 3, vt);
      const uint32_t m = pos[3] & ((1u << 30) - 1), margin = 5 * F + 6;
      exact = m < margin || m > (1u << 30) - 1 - margin;
    }
    if (exact) rns_exact_s<MAXF, MAXT>(&s, r, F, vlo, vhi, pos);
    w_sign = (pos[7] >> 31) != 0;
    if (w_sign) {
      uint32_t nw[8];
#pragma unroll
      for (int k = 0; k < 8; k++) nw[k] = ~pos[k];
      shr_words(nw, 8, 126, &wlo, &whi);
      wlo += 1;
      whi += (wlo == 0);
      wlo = (wlo >> 1) | (whi << 63);
      whi >>= 1;
    } else {
      shr_words(pos, 8, 126, &wlo, &whi);
      const uint64_t odd = wlo & 1;
      wlo = (wlo >> 1) | (whi << 63);
      whi >>= 1;
      wlo += odd;
      whi += (wlo < odd);
    }
  }

  // scaler.rs:316-351. Above 8 source moduli the output loop stays
  // rolled: unrolling it as well made the kernel body overflow the
  // instruction cache (ncu: a third of the stall cycles waiting for
  // instructions); its constants are then read with an indexed constant-bank
  // load per term. Smaller bodies run faster unrolled.
  constexpr int kOutUnroll = MAXF > 8 ? 1 : MAXT;
  // v <= 32 * 2^62 (at most 32 sources, each residue below 2^62), so
  // v * gamma = (v mod 2^62) * gamma + (v >> 62) * (gamma * 2^62 mod q_j):
  // two exact terms of the 128-bit sum below, and v needs no reduction
  // modulo each q_j. The sum then holds at most 15 terms below 2^124 (and a
  // few small ones) between reductions: below 2^128.
  if constexpr (TC) {
    // Every output pass done (split: passes 2 and 3) before the outputs, which
    // may go to the stage buffer that A overlays.
    if constexpr (!SPLIT) {
      if (!mbar_wait(bar_mma + 8, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
    } else {
      if (!mbar_wait(bar_mma + 16, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
      if (!mbar_wait(bar_mma + 24, 0, kTcWaitTries)) atomicAdd(&g_tc_wait_failures, 1u);
    }
    tc_fence_after();
  }
  const uint64_t v_low = vlo & ((1ull << 62) - 1);
  const uint64_t v_top = (vlo >> 62) | (vhi << 2);
  uint64_t* dst = out.at(poly, 0) + i;
#pragma unroll kOutUnroll
  for (int o = 0; o < MAXT; o++) {
    if (o < (int)s.out_len) {
      DevPrime pr;
      pr.p = s.p[o];
      pr.p2 = 2 * s.p[o];
      pr.bhi = s.bhi[o];
      pr.blo = s.blo[o];
      uint64_t y;
      if constexpr (EXACT) {
        // Every term below 2^62 q_j (r_k, v_low < 2^62; v_top < 32), so 14
        // products and the two gamma terms keep hi below 4 q_j.
        uint64_t lo = 0, hi = 0, acc = 0;
        if constexpr (TC) {
          // The output's sum below 2^81 (8 bytes of sums below 2^24), so hi
          // stays below 4 q_j with the gamma terms for q_j above 2^20.
          uint32_t c[8], w2[2];
          const uint32_t col = !SPLIT ? 8 * o : (uint32_t)o < tc.chunk ? 64 + 8 * o : 8 * (o - tc.chunk);
          tc_ld8(lane + col, c);
          tc_words<(MAXF <= 16)>(c, acc, w2);
          lo = join(w2[0], w2[1]);
          hi = acc;
          acc = 0;
        }
        mac128(hi, lo, v_low, s.gamma_neg[o]);
        mac128(hi, lo, v_top, s.gamma_neg_hi[o]);
        if constexpr (!TC) {
#pragma unroll
          for (int k = 0; k < MAXF; k++) {
            if (k < (int)F) {
              mac128(hi, lo, r[k], s.omega[o][k]);
              if ((k % 14) == 13) {
                acc = csub(acc + mont_fold(hi, lo, pr.p, s.pinv[o]), pr.p);
                hi = lo = 0;
              }
            }
          }
        }
        y = csub(acc + mont_fold(hi, lo, pr.p, s.pinv[o]), pr.p);
        if (!s.is_one) {
          // whi < 2^63: w mod q_j = whi * 2^64 + wlo in [0, 2q_j) from one
          // Shoup product and a reduction of wlo (conditional subtractions
          // when wlo < 8 q_j), where a 128-bit Barrett takes three times the
          // multiplies.
          const uint64_t lo_red = s.wbig ? csub(csub(csub(wlo, 2 * pr.p2), pr.p2), pr.p)
                                         : csub(mul_shoup_lazy(wlo, 1, s.one_shoup[o], pr.p), pr.p);
          const uint64_t wj = csub(mul_shoup_lazy(whi, s.r64[o], s.r64_shoup[o], pr.p), pr.p) + lo_red;
          y = csub(csub(y + (w_sign ? pr.p2 - wj : wj), pr.p2), pr.p);
        }
      } else {
        uint64_t lo = 0, hi = 0;
        if (!s.is_one) {
          const uint64_t wj = reduce128_lazy(whi, wlo, pr);
          lo = w_sign ? pr.p2 - wj : wj;
        }
        mac128(hi, lo, v_low, s.gamma_neg[o]);
        mac128(hi, lo, v_top, s.gamma_neg_hi[o]);
#pragma unroll
        for (int k = 0; k < MAXF; k++) {
          if (k < (int)F) {
            mac128(hi, lo, r[k], s.omega[o][k]);
            if ((k % 14) == 13) {  // keep the exact sum below 2^128
              lo = reduce128(hi, lo, pr);
              hi = 0;
            }
          }
        }
        y = reduce128(hi, lo, pr);
      }
      if constexpr (TOP > 0) {
        if (fwd_here || dig_here)
          scale_stage<(MAXF > MAXT ? MAXF : MAXT) * 128, TC>()[(o * (1 << TOP) + t) * G + gi] = y;
        else dst[(uint64_t)o << logn] = y;
      } else {
        dst[(uint64_t)o << logn] = y;
      }
    }
  }
  if constexpr (TC) {
    // Every lane's reads are done (tc_ld8 waits for them): free the columns.
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 1) tc_dealloc(tmem, tc.cols);
  }
  if constexpr (TOP > 0) {
    if (fwd_here || dig_here) {
      __syncthreads();
      const uint64_t* staged = scale_stage<(MAXF > MAXT ? MAXF : MAXT) * 128, TC>();
      if (fwd_here) {
        for (uint32_t item = threadIdx.x; item < s.out_len * G; item += 128) {
          const uint32_t o = item / G, g2 = item % G;
          uint64_t x[1 << TOP];
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) x[u] = staged[(o * (1 << TOP) + u) * G + g2];
          fwd_top_stages<TOP>(x, fe.primes[o]);
          uint64_t* row = out.at(poly, o) + b0 + g2;
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) row[(uint64_t)u << logb] = x[u];
        }
      } else {
        // Digit d (output limb d) in key limb j: key_switching_key.rs:227-235
        // with rq/mod.rs:518-540, the first forward stages of its transform.
        const uint32_t per_digit = fe.digit_limbs * G;
        const uint32_t pbase = (poly / fe.period) * s.out_len;
        for (uint32_t item = threadIdx.x; item < s.out_len * per_digit; item += 128) {
          const uint32_t d = item / per_digit, rem = item - d * per_digit;
          const uint32_t j = rem / G, g2 = rem % G;
          const DevPrime kp = fe.digit_primes[j];
          uint64_t x[1 << TOP];
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) {
            const uint64_t v = staged[(d * (1 << TOP) + u) * G + g2];
            x[u] = fe.digit_raw ? v : reduce64_lazy(v, kp);
          }
          fwd_top_stages<TOP>(x, kp);
          uint64_t* row = fe.digits.at(pbase + d, j) + b0 + g2;
#pragma unroll
          for (int u = 0; u < (1 << TOP); u++) row[(uint64_t)u << logb] = x[u];
        }
      }
    }
  }
}

static std::atomic<bool> g_rns_tc{true};
bool rns_tc_enabled() { return g_rns_tc.load(std::memory_order_relaxed); }
void set_rns_tc(bool on) { g_rns_tc.store(on, std::memory_order_relaxed); }

uint64_t rns_tc_wait_failures() {
  uint32_t v = 0;
  check_cuda(cudaMemcpyFromSymbol(&v, g_tc_wait_failures, sizeof(v)), "cudaMemcpyFromSymbol");
  return v;
}

// 228 KB of shared memory per SM over its 512 tensor-memory columns.
constexpr size_t kTcSmemPerColumn = 233472 / 512;

// Once per tensor-core kernel and device: reads the kernel's static shared
// memory and raises its dynamic limit to cover its largest operands
// (`operands` bytes) and the floor of a 128-column CTA. Returns the static
// shared memory.
static size_t tc_prepare(const void* kern, size_t operands) {
  struct Entry {
    const void* kern;
    int dev;
    size_t stat;
  };
  static std::mutex mu;
  static std::vector<Entry> done;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lock(mu);
  for (const Entry& e : done)
    if (e.kern == kern && e.dev == dev) return e.stat;
  cudaFuncAttributes a{};
  check_cuda(cudaFuncGetAttributes(&a, kern), "cudaFuncGetAttributes");
  const size_t limit = std::max<size_t>(operands, 128 * kTcSmemPerColumn - 1024 - a.sharedSizeBytes);
  check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit),
             "cudaFuncSetAttribute");
  done.push_back(Entry{kern, dev, a.sharedSizeBytes});
  return a.sharedSizeBytes;
}

template <int MAXF, int MAXT, bool EXACT = false, int TOP = 0>
void launch_rns_scale(const RnsScalerD& sc, uint32_t logn, PolyRef in, PolyRef out, uint32_t start,
                      uint32_t out_len, uint64_t total, cudaStream_t st, const InverseTop* top = nullptr,
                      const ForwardTop* fwd = nullptr) {
  const RnsScalerHost& h = sc.host;
  const size_t F = h.from_len;
  for (uint32_t first = 0; first < out_len; first += MAXT) {
    const uint32_t n = std::min<uint32_t>(MAXT, out_len - first);
    RnsLaunch<MAXF, MAXT> s;
    memset(&s, 0, sizeof(s));
    s.from_len = (uint32_t)F;
    s.out_len = n;
    s.is_one = h.is_one ? 1 : 0;
    s.shift = (uint32_t)h.theta_garner_shift;
    s.tg_sign = h.theta_gamma_sign ? 1 : 0;
    s.tg_lo = h.theta_gamma_lo;
    s.tg_hi = h.theta_gamma_hi;
    for (size_t k = 0; k < F; k++) {
      s.tgar_lo[k] = h.theta_garner_lo[k];
      s.tgar_hi[k] = h.theta_garner_hi[k];
      s.to_lo[k] = h.theta_omega_lo[k];
      s.to_hi[k] = h.theta_omega_hi[k];
      if (h.theta_omega_sign[k]) s.to_sign |= 1u << k;
    }
    if (EXACT && !sc.mont) throw Error(FHEG_ERR_INTERNAL, "Montgomery scaling needs odd target moduli");
    s.wbig = 1;
    for (uint32_t o = 0; o < n; o++) {
      const size_t j = start + first + o;
      if (EXACT) {
        for (size_t k = 0; k < F; k++) s.omega[o][k] = sc.omega_mont[j * F + k];
        s.gamma_neg[o] = sc.gamma_neg_mont[j];
        s.gamma_neg_hi[o] = sc.gamma_neg_hi_mont[j];
        s.pinv[o] = sc.to_pinv[j];
        const uint64_t q = sc.to_moduli[j];
        s.r64[o] = (uint64_t)(((unsigned __int128)1 << 64) % q);
        s.r64_shoup[o] = shoup(s.r64[o], q);
        s.one_shoup[o] = shoup(1, q);
        if (q <= (1ull << 61)) s.wbig = 0;
      } else {
        for (size_t k = 0; k < F; k++) s.omega[o][k] = h.omega[j * F + k];
        s.gamma_neg[o] = sc.gamma_neg[j];
        s.gamma_neg_hi[o] = sc.gamma_neg_hi[j];
      }
      s.p[o] = sc.to_moduli[j];
      s.bhi[o] = sc.to_bhi[j];
      s.blo[o] = sc.to_blo[j];
    }
    PolyRef o = out;
    o.base += (uint64_t)first << logn;
    FwdEpilogue fe{};
    if (fwd) {
      if (fwd->digit_primes && first > 0) throw Error(FHEG_ERR_INTERNAL, "digit expansion needs one launch");
      fe = FwdEpilogue{fwd->primes + first, fwd->period, fwd->take, fwd->digit_primes, fwd->digit_limbs,
                       fwd->digit_raw, fwd->digits};
    }
    const unsigned threads = 128;
    // The tensor-core form from 12 source moduli: with fewer, its carries
    // cost about what the multiplies they replace did, and its shared memory
    // halves the CTAs per SM (6 sources: 0.40 against 0.33 ms on GB300).
    if constexpr (EXACT && MAXF >= 12 && MAXF <= 32) {
      const uint32_t head = h.is_one ? 3 : 7;
      const uint32_t n0 = (8 * head + 15) / 16 * 16, n1 = (8 * n + 15) / 16 * 16;
      if (sc.tc_mat.ptr && rns_tc_enabled() && n1 <= 128 && (TOP > 0 || total % 128 == 0)) {
        constexpr uint32_t KP = (8 * MAXF + 15) / 16 * 16;
        if (sc.tc_kp != KP) throw Error(FHEG_ERR_INTERNAL, "tensor-core scaler matrix of another width");
        auto kern = k_rns_scale<MAXF, MAXT, EXACT, TOP, false, true>;
        // The stage buffer (TOP > 0) overlaid by A, then B (the larger pass).
        constexpr size_t kStage = TOP > 0 ? (size_t)(MAXF > MAXT ? MAXF : MAXT) * 128 * 8 : 0;
        constexpr size_t kBOff = ((128 * KP * 2 > kStage ? 128 * KP * 2 : kStage) + 127) / 128 * 128;
        const size_t stat = tc_prepare(reinterpret_cast<const void*>(kern), kBOff + 128 * 2 * KP);
        // Shared memory of a form (operand buffer of `rows` rows), at least
        // cols * 456 bytes with the 1 KB the SM reserves per CTA: the SM's
        // 228 KB then never holds CTAs asking for more than its 512
        // tensor-memory columns. CTAs per SM of a form by shared and tensor
        // memory.
        auto dyn_of = [&](uint32_t rows, uint32_t cols) {
          return std::max<size_t>(kBOff + (size_t)rows * 2 * KP, cols * kTcSmemPerColumn - 1024 - stat);
        };
        auto ctas = [&](size_t dyn, uint32_t cols) {
          return std::min<size_t>(233472 / (dyn + stat + 1024), 512 / cols);
        };
        uint32_t cols = std::max(n0, n1) <= 64 ? 64 : 128;
        size_t dyn = dyn_of(std::max(n0, n1), cols);
        TcMat tc{static_cast<const uint16_t*>(sc.tc_mat.ptr), KP, head, 7 + start + first, n0, n1, cols,
                 (uint32_t)kBOff, 0, 0};
        // The split form (scale-downs of two outputs or more) where it fits
        // more CTAs on an SM. Only a wide A (over 16 sources) leaves it room
        // to: with fewer, 64 columns or the same count of CTAs hold already.
        if constexpr (MAXT > 8 && MAXF > 16) {
          if (!h.is_one && n >= 2) {
            const uint32_t chunk = (n + 1) / 2, s1 = (8 * chunk + 15) / 16 * 16, s2 = (8 * (n - chunk) + 15) / 16 * 16;
            auto skern = k_rns_scale<MAXF, MAXT, EXACT, TOP, false, true, true>;
            const size_t sstat = tc_prepare(reinterpret_cast<const void*>(skern), kBOff + 128 * 2 * KP);
            const size_t sdyn = std::max<size_t>(kBOff + (size_t)std::max(32u, s1) * 2 * KP,
                                                 128 * kTcSmemPerColumn - 1024 - sstat);
            if (s1 <= 64 && std::min<size_t>(233472 / (sdyn + sstat + 1024), 4) > ctas(dyn, cols)) {
              tc.n0 = 32;
              tc.n1 = s1;
              tc.n2 = s2;
              tc.chunk = chunk;
              tc.cols = 128;
              skern<<<blocks_for(total, threads), threads, sdyn, st>>>(
                  s, logn, in, o, total, top ? top->primes : nullptr, top ? top->mont : 0u, fe, tc);
              after_launch("k_rns_scale");
              continue;
            }
          }
        }
        kern<<<blocks_for(total, threads), threads, dyn, st>>>(s, logn, in, o, total, top ? top->primes : nullptr,
                                                              top ? top->mont : 0u, fe, tc);
        after_launch("k_rns_scale");
        continue;
      }
    }
    // The kept-high-word sums for the source counts of the default
    // extensions (L = 3, 6, 12); correct for any scaler, faster for these.
    constexpr bool kFastV = EXACT && (MAXF == 3 || MAXF == 6 || MAXF == 12);
    k_rns_scale<MAXF, MAXT, EXACT, TOP, kFastV, false><<<blocks_for(total, threads), threads, 0, st>>>(
        s, logn, in, o, total, top ? top->primes : nullptr, top ? top->mont : 0u, fe, TcMat{});
    after_launch("k_rns_scale");
  }
}

template <int MAXF, int MAXT>
static void launch_rns_scale_top(const RnsScalerD& s, uint32_t logn, PolyRef in, PolyRef out, uint32_t start,
                                 uint32_t out_len, uint64_t total, cudaStream_t st, const InverseTop& top,
                                 const ForwardTop* fwd) {
  switch (top.s1) {
    case 1: launch_rns_scale<MAXF, MAXT, true, 1>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    case 2: launch_rns_scale<MAXF, MAXT, true, 2>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    case 3: launch_rns_scale<MAXF, MAXT, true, 3>(s, logn, in, out, start, out_len, total, st, &top, fwd); break;
    default: throw Error(FHEG_ERR_INTERNAL, "unsupported strided stage count");
  }
}

bool rns_scale_takes_top(const RnsScalerD& s, uint32_t logn, uint32_t out_len, uint32_t s1) {
  const size_t F = s.host.from_len;
  const bool exact = (F == 6 || F == 13 || F == 3 || F == 7) ? out_len <= 8 : (F == 12 || F == 25) && out_len <= 16;
  return exact && s.mont && s1 >= 1 && s1 <= 3 && logn >= 7;
}

void rns_scale(const RnsScalerD& s, uint32_t logn, PolyRef in, PolyRef out, uint32_t start, uint32_t out_len,
               uint64_t polys, cudaStream_t st, const InverseTop* top, const ForwardTop* fwd) {
  const uint64_t total = polys << logn;
  if (total == 0 || out_len == 0) return;
  const size_t F = s.host.from_len;
  if (fwd && (!top || fwd->s1 != top->s1))
    throw Error(FHEG_ERR_INTERNAL, "forward strided stages need the same count of inverse ones");
  if (top) {
    if (!rns_scale_takes_top(s, logn, out_len, top->s1))
      throw Error(FHEG_ERR_INTERNAL, "RNS scaling cannot apply these strided stages");
    if (F == 6) launch_rns_scale_top<6, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 13) launch_rns_scale_top<13, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 3) launch_rns_scale_top<3, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 7) launch_rns_scale_top<7, 8>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else if (F == 12) launch_rns_scale_top<12, 16>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    else launch_rns_scale_top<25, 16>(s, logn, in, out, start, out_len, total, st, *top, fwd);
    return;
  }
  // Exact source counts of the default multiplications at L = 3, 6, 12
  // (extension from L, scale-down from 2L + 1), odd target moduli.
  if (!s.mont) {
    if (F <= 8) launch_rns_scale<8, 8>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 16 && out_len <= 8) launch_rns_scale<16, 8>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 16) launch_rns_scale<16, 16>(s, logn, in, out, start, out_len, total, st);
    else if (F <= 32) launch_rns_scale<32, 16>(s, logn, in, out, start, out_len, total, st);
    else throw Error(FHEG_ERR_UNSUPPORTED, "RNS scaling from more than 32 moduli is not supported");
    return;
  }
  if (F == 6 && out_len <= 8) launch_rns_scale<6, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 13 && out_len <= 8) launch_rns_scale<13, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 3 && out_len <= 8) launch_rns_scale<3, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 7 && out_len <= 8) launch_rns_scale<7, 8, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 12 && out_len <= 16) launch_rns_scale<12, 16, true>(s, logn, in, out, start, out_len, total, st);
  else if (F == 25 && out_len <= 16) launch_rns_scale<25, 16, true>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 8) launch_rns_scale<8, 8>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 16 && out_len <= 8) launch_rns_scale<16, 8>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 16) launch_rns_scale<16, 16>(s, logn, in, out, start, out_len, total, st);
  else if (F <= 32) launch_rns_scale<32, 16>(s, logn, in, out, start, out_len, total, st);
  else throw Error(FHEG_ERR_UNSUPPORTED, "RNS scaling from more than 32 moduli is not supported");
}

RnsScalerD::RnsScalerD(const Context& from, const Context& to, const BigUint& num, const BigUint& den)
    : host(make_rns_scaler(*from.rns, *to.rns, num, den)) {
  const size_t T = host.to_len;
  gamma_neg.resize(T);
  gamma_neg_hi.resize(T);
  to_moduli = to.moduli;
  to_bhi.resize(T);
  to_blo.resize(T);
  for (size_t j = 0; j < T; j++) {
    gamma_neg[j] = (to.moduli[j] - host.gamma[j]) % to.moduli[j];
    gamma_neg_hi[j] = mulmod(gamma_neg[j], (1ull << 62) % to.moduli[j], to.moduli[j]);
    barrett128(to.moduli[j], &to_bhi[j], &to_blo[j]);
  }
  mont = true;
  for (size_t j = 0; j < T; j++) mont = mont && (to.moduli[j] & 1);
  if (mont) {
    const size_t F = host.from_len;
    omega_mont.resize(T * F);
    gamma_neg_mont.resize(T);
    gamma_neg_hi_mont.resize(T);
    to_pinv.resize(T);
    for (size_t j = 0; j < T; j++) {
      const uint64_t q = to.moduli[j];
      const uint64_t r = (uint64_t)(((unsigned __int128)1 << 64) % q);
      for (size_t k = 0; k < F; k++) omega_mont[j * F + k] = mulmod(host.omega[j * F + k], r, q);
      gamma_neg_mont[j] = mulmod(gamma_neg[j], r, q);
      gamma_neg_hi_mont[j] = mulmod(gamma_neg_hi[j], r, q);
      uint64_t inv = q;  // q^-1 mod 2^64 by Newton's iteration
      for (int it = 0; it < 6; it++) inv *= 2 - q * inv;
      to_pinv[j] = 0 - inv;
    }
    build_tc_matrix();
  }
}

// FP16 bit pattern of an integer 0..255 (exact).
static uint16_t half_bits(uint32_t v) {
  if (v == 0) return 0;
  int e = 31 - __builtin_clz(v);
  return (uint16_t)(((e + 15) << 10) | ((v << (10 - e)) & 0x3FF));
}

// The byte matrix of the tensor-core form (k_rns_scale, TC): for source k and
// byte b (column 8k + b), rows 0-23 hold the bytes of theta_garner_k 2^(8b),
// rows 24-55 those of (+/- theta_omega_k) 2^(8b) mod 2^256, and rows 56 + 8j ..
// 56 + 8j + 7 those of omega_jk 2^64 2^(8b) mod q_j; FP16 values in the
// operand layout of tc.cuh (groups of 8 rows, 16 * kp bytes each). Built for
// up to 32 source moduli with every target modulus above 2^20.
void RnsScalerD::build_tc_matrix() {
  const size_t F = host.from_len, T = host.to_len;
  if (!mont || F == 0 || F > 32) return;
  for (uint64_t q : to_moduli)
    if (q <= (1ull << 20)) return;
  const uint32_t kp = (uint32_t)((8 * F + 15) / 16 * 16);
  std::vector<uint16_t> m((7 + T) * 8 * kp, 0);
  auto put = [&](size_t row, size_t k, uint32_t byte) {
    const size_t off = (row & 7) * 16 + (k & 7) * 2 + (k >> 3) * 128 + (row >> 3) * 16 * kp;
    m[off / 2] = half_bits(byte);
  };
  for (size_t k = 0; k < F; k++) {
    const uint64_t tg[2] = {host.theta_garner_lo[k], host.theta_garner_hi[k]};
    for (uint32_t b = 0; b < 8; b++) {
      const size_t col = 8 * k + b;
      for (uint32_t c = 0; c < 24; c++) {
        const int idx = (int)c - (int)b;
        put(c, col, idx >= 0 && idx < 16 ? (uint32_t)(tg[idx / 8] >> (8 * (idx % 8))) & 255 : 0);
      }
      uint64_t x[4] = {0, 0, 0, 0};  // theta_omega_k << 8b, 256 bits
      const uint64_t lo = host.theta_omega_lo[k], hi = host.theta_omega_hi[k];
      x[0] = b ? lo << (8 * b) : lo;
      x[1] = b ? (hi << (8 * b)) | (lo >> (64 - 8 * b)) : hi;
      x[2] = b ? hi >> (64 - 8 * b) : 0;
      if (host.theta_omega_sign[k]) {
        bool carry = true;
        for (int w = 0; w < 4; w++) {
          x[w] = ~x[w] + (carry ? 1 : 0);
          carry = carry && x[w] == 0;
        }
      }
      for (uint32_t c = 0; c < 32; c++) put(24 + c, col, (uint32_t)(x[c / 8] >> (8 * (c % 8))) & 255);
      for (size_t j = 0; j < T; j++) {
        const uint64_t q = to_moduli[j];
        const uint64_t p2 = (uint64_t)(((unsigned __int128)1 << (8 * b)) % q);
        const uint64_t v = mulmod(omega_mont[j * F + k], p2, q);
        for (uint32_t c = 0; c < 8; c++) put(56 + 8 * j + c, col, (uint32_t)(v >> (8 * c)) & 255);
      }
    }
  }
  tc_mat.alloc(m.size() * sizeof(uint16_t));
  upload(tc_mat.ptr, m.data(), m.size() * sizeof(uint16_t));
  tc_kp = kp;
}

Scaler::Scaler(std::shared_ptr<Context> f, std::shared_ptr<Context> t, const BigUint& n, const BigUint& d)
    : from(std::move(f)), to(std::move(t)), num(n), den(d) {
  if (from->degree != to->degree) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Incompatible degrees");
  rns.reset(new RnsScalerD(*from, *to, num, den));
  number_common_moduli = 0;
  if (rns->host.is_one) {  // rq/scaler.rs:32-40
    while (number_common_moduli < from->L() && number_common_moduli < to->L() &&
           from->moduli[number_common_moduli] == to->moduli[number_common_moduli])
      number_common_moduli++;
  }
}

}  // namespace fheg
