// Batched negacyclic NTT kernels for sm_103a.
//
// The transforms compute exactly what fhe-math/src/ntt/native.rs computes:
//   forward  (77-102):  Cooley-Tukey, bit-reversed output, Shoup twiddles
//                       omegas[m + chunk] at the stage with m chunks;
//   backward (106-132): Gentleman-Sande with zetas_inv[N - 2m + chunk],
//                       then multiplication by N^-1.
// Residues stay in Harvey's lazy ranges ([0, 4p) forward, [0, 2p) inverse)
// and are reduced at the end, so outputs are bit-identical to the reference.
//
// Layout: one CTA transforms one block of 2^bl residues of one limb (bl <= 14,
// resident in shared memory). Each thread keeps 16 residues in registers
// (32 in blocks below 2^12) and runs up to four (five) butterfly stages on
// them per round; rounds exchange data through shared memory with an XOR
// swizzle that keeps 64-bit
// accesses free of bank conflicts. A transform of 2^logn is either one block
// (bl = logn) or, following the plan of ntt_block_logn(), a strided pass over
// groups of 2^(logn - bl) elements for the first (forward) or last (inverse)
// stages plus the block kernel for the others.
//
// The kernels are templates over a source functor (produces the input
// residue of element i; fuses element-wise prologues such as the BFV tensor
// product) and a destination functor (consumes the output; fuses epilogues
// such as the key-switching inner product).
#pragma once

#include <algorithm>

#include "common.cuh"

namespace fheg {
// Internal linkage: every translation unit that includes this header gets its
// own kernels and launch helpers (a template kernel instantiated in two units
// must not share one host-side registration or attribute flag).
namespace {

// Job decoding shared by all NTT kernels: blockIdx.x enumerates
// (poly, limb, block) with block fastest.
// With `jobs` set, the launch is ragged: unit u is jobs[u] = (poly, limb,
// aux, -) instead of (u / limbs, u % limbs, 0), so one launch can cover
// polynomials with different numbers of limbs (ciphertexts at different
// levels). `limb` always indexes `primes`.
struct NttGeom {
  const DevPrime* primes;  // one entry per limb (modulus index)
  uint32_t limbs;          // limbs per polynomial (1 for ragged launches)
  uint32_t s1;             // stages handled by the strided pass (0 to 4)
  const uint4* jobs;       // optional ragged job table
  uint32_t mont;           // inverse transforms: inputs carry a factor 2^-64 (Montgomery products)
  uint32_t pf_stride;      // > 0: each CTA prefetches into L2 the input of CTA blockIdx.x + pf_stride
};


// Final scale of an inverse transform: N^-1, or N^-1 * 2^64 when the inputs
// are Montgomery products (a * b * 2^-64), which cancels their factor.
__device__ __forceinline__ uint64_t inv_final_scale(const NttGeom& g, const DevPrime& pr, uint64_t v) {
  return g.mont ? mul_shoup(v, pr.ninv_mont, pr.ninv_mont_shoup, pr.p) : mul_shoup(v, pr.ninv, pr.ninv_shoup, pr.p);
}

// Sources that load their inputs themselves through shared memory declare
// kStaged = true and provide stage<LOGN, T, E>(job, prime, base, sm, tid, x),
// which fills x[e] with the value of element base + tid + e * T and leaves the
// shared buffer free (ending with a barrier).
template <class S>
constexpr auto src_is_staged(int) -> decltype(S::kStaged) {
  return S::kStaged;
}
template <class S>
constexpr bool src_is_staged(long) {
  return false;
}

// Sources whose values are Montgomery products declare kMontgomery = true.
template <class S>
constexpr auto src_is_montgomery(int) -> decltype(S::kMontgomery) {
  return S::kMontgomery;
}
template <class S>
constexpr bool src_is_montgomery(long) {
  return false;
}

struct NttJob {
  uint32_t poly, limb, beta, aux;
};

// L2 prefetch hint (no fault, no register result).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Sources that can name the addresses they will read declare
// prefetch(job, i): a hint for element i of that job.
template <class S>
__device__ __forceinline__ auto src_prefetch(const S& s, const NttJob& j, uint32_t i, int)
    -> decltype(s.prefetch(j, i), void()) {
  s.prefetch(j, i);
}
template <class S>
__device__ __forceinline__ void src_prefetch(const S&, const NttJob&, uint32_t, long) {}



__device__ __forceinline__ NttJob unit_job(const NttGeom& g, uint32_t unit) {
  NttJob j;
  if (g.jobs) {
    const uint4 t = g.jobs[unit];
    j.poly = t.x;
    j.limb = t.y;
    j.aux = t.z;
  } else {
    j.limb = unit % g.limbs;
    j.poly = unit / g.limbs;
    j.aux = 0;
  }
  j.beta = 0;
  return j;
}

__device__ __forceinline__ NttJob decode_job_at(const NttGeom& g, uint32_t block) {
  uint32_t job = block;
  const uint32_t beta = job & ((1u << g.s1) - 1);
  NttJob j = unit_job(g, job >> g.s1);
  j.beta = beta;
  return j;
}

// Block-pass kernels: while this CTA works, the CTA that will take its place
// on the SM (about pf_stride blocks later) gets its input rows pulled into L2,
// one hint per 128-byte line, so its load phase hits L2 instead of DRAM.
template <int LOGN, int T, class Src>
__device__ __forceinline__ void prefetch_next(const NttGeom& g, const Src& src, uint32_t tid) {
  if (!g.pf_stride) return;
  const uint32_t nb = blockIdx.x + g.pf_stride;
  if (nb >= gridDim.x) return;
  const NttJob jn = decode_job_at(g, nb);
  const uint32_t base = jn.beta << LOGN;
  for (uint32_t k = tid * 16; k < (1u << LOGN); k += T * 16) src_prefetch(src, jn, base + k, 0);
}

__device__ __forceinline__ NttJob decode_job(const NttGeom& g) {
  uint32_t job = blockIdx.x;
  const uint32_t beta = job & ((1u << g.s1) - 1);
  NttJob j = unit_job(g, job >> g.s1);
  j.beta = beta;
  return j;
}

// Shared-memory swizzle: the low 4 bits of the word index are XORed with
// bits 4-7 and 5-8. Every access pattern of the rounds below (and of the
// coalesced staging) then maps the 16 threads of a half warp to 16 distinct
// 8-byte bank pairs, for every supported size.
__host__ __device__ __forceinline__ constexpr uint32_t swz(uint32_t i) { return i ^ ((i >> 4) & 15) ^ ((i >> 5) & 15); }

// The swizzle is linear over GF(2): swz(a ^ b) = swz(a) ^ swz(b). Every
// shared-memory index of the kernels below is the bitwise OR of a part that
// depends on the thread and a compile-time part with disjoint bits, so an
// access costs one XOR of the thread's swizzled byte offset with a constant
// (instead of shifts, masks and XORs per access).
__device__ __forceinline__ uint64_t& sm_at(uint64_t* sm, uint32_t off8) {
  return *reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(sm) + off8);
}
// Byte offset of the swizzled word index i.
__host__ __device__ __forceinline__ constexpr uint32_t swz8(uint32_t i) { return swz(i) << 3; }

// Residues per thread: 16 (radix-16 rounds) in blocks of 2^12 to 2^14, 32
// (radix-32 rounds) in smaller blocks. With 32 residues the 2^12-2^14 kernels
// spilled 100-470 bytes per thread at their 128-register budget; with 16 they
// spill nothing at 128. Blocks of 2^12 (256 threads) run three CTAs per SM
// under an 80-register cap (24 warps, a few words spilled). On GB300 the
// forward + inverse NTT at N = 2^14 with 2^12 blocks went from 1,064 GB/s
// (32 residues) to 1,209 GB/s; four CTAs under 64 registers spilled more and
// reached 1,150, and 8 residues per thread (512 threads, two CTAs, radix-8
// rounds) 1,131.
template <int LOGN>
struct NttShape {
  static constexpr int LOGE = LOGN < 5 ? LOGN : (LOGN >= 12 ? 4 : 5);
  static constexpr int E = 1 << LOGE;
  static constexpr int N = 1 << LOGN;
  static constexpr int T = N / E;
  // Blocks per SM the register budget must allow: 3 for 2^12 blocks, else
  // at least 512 threads' worth (a 128-register budget).
  static constexpr int MIN_BLOCKS = LOGN == 12 ? 3 : (T >= 512 ? 1 : (512 / T > 32 ? 32 : 512 / T));
};

// One forward round: global stages S0 .. S0+K-1 of a transform of size 2^LOGN
// held as E residues per thread (E / 2^K groups of 2^K). Group g holds
// elements c * 2^(LOGN-S0) + b + t * 2^(LOGN-S0-K) for t < 2^K. The stage
// with 2^s chunks uses omegas[2^s * tw_mult + chunk] (tw_mult = 1 for a whole
// transform); the 2^r twiddles a group needs at round stage r are contiguous.
template <int LOGN, int S0, int K>
__device__ __forceinline__ void fwd_round(uint64_t* x, uint32_t tid, const DevPrime& pr, uint32_t tw_mult) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  constexpr int G = E >> K;
  constexpr int LMIN_LOG = LOGN - S0 - K;
#pragma unroll
  for (int q = 0; q < G; q++) {
    const uint32_t g = tid + q * T;
    const uint32_t c = g >> LMIN_LOG;
    uint64_t* xx = x + q * (1 << K);
#pragma unroll
    for (int r = 0; r < K; r++) {
      const int half = 1 << (K - 1 - r);
      const ulonglong2* twr = pr.tw + (1u << (S0 + r)) * tw_mult + (c << r);
      // Constant trip counts at every level keep x[] in registers.
#pragma unroll
      for (int t = 0; t < (1 << K); t++) {
        if (t & half) continue;
        const ulonglong2 w = __ldg(twr + (t >> (K - r)));
        fwd_bfly(xx[t], xx[t + half], w.x, w.y, pr.p, pr.p2);
      }
    }
  }
}

// Index of element (q, t) of a forward round. Since tid < T (a power of
// two), g = tid | q*T and the result is fwd_index(tid, 0, 0) | fwd_index(0,
// q, t) with disjoint bits.
template <int LOGN, int S0, int K>
__host__ __device__ __forceinline__ constexpr uint32_t fwd_index(uint32_t tid, int q, int t) {
  constexpr int T = NttShape<LOGN>::T;
  constexpr int LMIN_LOG = LOGN - S0 - K;
  const uint32_t g = tid + q * T;
  const uint32_t c = g >> LMIN_LOG;
  const uint32_t b = g & ((1u << LMIN_LOG) - 1);
  return (c << (LOGN - S0)) + b + ((uint32_t)t << LMIN_LOG);
}

template <int LOGN, int S0, int K>
__device__ __forceinline__ void fwd_to_smem(const uint64_t* x, uint64_t* sm, uint32_t tid) {
  constexpr int E = NttShape<LOGN>::E;
  const uint32_t base = swz8(fwd_index<LOGN, S0, K>(tid, 0, 0));
#pragma unroll
  for (int e = 0; e < E; e++) sm_at(sm, base ^ swz8(fwd_index<LOGN, S0, K>(0, e >> K, e & ((1 << K) - 1)))) = x[e];
}

template <int LOGN, int S0, int K>
__device__ __forceinline__ void fwd_from_smem(uint64_t* x, uint64_t* sm, uint32_t tid) {
  constexpr int E = NttShape<LOGN>::E;
  const uint32_t base = swz8(fwd_index<LOGN, S0, K>(tid, 0, 0));
#pragma unroll
  for (int e = 0; e < E; e++) x[e] = sm_at(sm, base ^ swz8(fwd_index<LOGN, S0, K>(0, e >> K, e & ((1 << K) - 1))));
}

// Applies forward rounds S0, S0+LOGE, ... up to LOGN, exchanging through smem.
template <int LOGN, int S0>
__device__ __forceinline__ void fwd_rounds(uint64_t* x, uint64_t* sm, uint32_t tid, const DevPrime& pr,
                                           uint32_t tw_mult) {
  constexpr int LOGE = NttShape<LOGN>::LOGE;
  constexpr int K = (LOGN - S0) < LOGE ? (LOGN - S0) : LOGE;
  fwd_round<LOGN, S0, K>(x, tid, pr, tw_mult);
  if constexpr (S0 + K < LOGN) {
    constexpr int K2 = (LOGN - S0 - K) < LOGE ? (LOGN - S0 - K) : LOGE;
    __syncthreads();
    fwd_to_smem<LOGN, S0, K>(x, sm, tid);
    __syncthreads();
    fwd_from_smem<LOGN, S0 + K, K2>(x, sm, tid);
    fwd_rounds<LOGN, S0 + K>(x, sm, tid, pr, tw_mult);
  } else {
    // Leave the output in shared memory for a coalesced store.
    __syncthreads();
    fwd_to_smem<LOGN, S0, K>(x, sm, tid);
    __syncthreads();
  }
}

// Forward NTT of blocks of 2^LOGN elements. With g.s1 > 0 the block is block
// `beta` of a transform of size 2^(LOGN + s1) whose first s1 stages already
// ran (ntt_fwd_top). REDUCE selects reduced ([0, p)) or lazy ([0, 4p)) output.
template <int LOGN, bool REDUCE, class Src, class Dst>
__global__ void __launch_bounds__(NttShape<LOGN>::T, NttShape<LOGN>::MIN_BLOCKS) k_ntt_fwd(NttGeom g, Src src, Dst dst) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  extern __shared__ uint64_t sm[];
  const uint32_t tid = threadIdx.x;
  const NttJob jb = decode_job(g);
  const DevPrime pr = g.primes[jb.limb];
  const uint32_t base = jb.beta << LOGN;
  prefetch_next<LOGN, T>(g, src, tid);
  uint64_t x[E];
  // Round 0 holds elements tid + e*T: coalesced loads.
#pragma unroll
  for (int e = 0; e < E; e++) x[e] = src(jb, pr, base + tid + e * T);
  fwd_rounds<LOGN, 0>(x, sm, tid, pr, (1u << g.s1) + jb.beta);
  const uint32_t sb = swz8(tid);
#pragma unroll
  for (int e = 0; e < E; e++) {
    const uint32_t i = tid + e * T;
    uint64_t v = sm_at(sm, sb ^ swz8(e * T));
    if (REDUCE) v = reduce4(v, pr.p, pr.p2);
    dst(jb, pr, base + i, v);
  }
}

// ---------------------------------------------------------------------------
// Inverse rounds: global GS stages with half-size l = 2^(U0+r), r < K.
// Group g = c * 2^U0 + b holds elements c * 2^(U0+K) + b + t * 2^U0.
template <int LOGN, int U0, int K>
__host__ __device__ __forceinline__ constexpr uint32_t inv_index(uint32_t tid, int q, int t) {
  constexpr int T = NttShape<LOGN>::T;
  const uint32_t g = tid + q * T;
  const uint32_t c = g >> U0;
  const uint32_t b = g & ((1u << U0) - 1);
  return (c << (U0 + K)) + b + ((uint32_t)t << U0);
}

template <int LOGN, int U0, int K>
__device__ __forceinline__ void inv_round(uint64_t* x, uint32_t tid, const DevPrime& pr, uint32_t n_total,
                                          uint32_t s1, uint32_t beta) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  constexpr int G = E >> K;
#pragma unroll
  for (int q = 0; q < G; q++) {
    const uint32_t g = tid + q * T;
    const uint32_t c = g >> U0;
    uint64_t* xx = x + q * (1 << K);
#pragma unroll
    for (int r = 0; r < K; r++) {
      // m_local = N_local / (2l) chunks of this block at this stage.
      const uint32_t m_local = 1u << (LOGN - 1 - U0 - r);
      const ulonglong2* twr = pr.itw + (n_total - (m_local << (s1 + 1)) + beta * m_local + (c << (K - 1 - r)));
      const int span = 1 << r;
#pragma unroll
      for (int t = 0; t < (1 << K); t++) {
        if (t & span) continue;
        const ulonglong2 z = __ldg(twr + (t >> (r + 1)));
        inv_bfly(xx[t], xx[t + span], z.x, z.y, pr.p, pr.p2);
      }
    }
  }
}

// As fwd_index: inv_index(tid, q, t) = inv_index(tid, 0, 0) | inv_index(0, q, t).
template <int LOGN, int U0, int K>
__device__ __forceinline__ void inv_to_smem(const uint64_t* x, uint64_t* sm, uint32_t tid) {
  constexpr int E = NttShape<LOGN>::E;
  const uint32_t base = swz8(inv_index<LOGN, U0, K>(tid, 0, 0));
#pragma unroll
  for (int e = 0; e < E; e++) sm_at(sm, base ^ swz8(inv_index<LOGN, U0, K>(0, e >> K, e & ((1 << K) - 1)))) = x[e];
}

template <int LOGN, int U0, int K>
__device__ __forceinline__ void inv_from_smem(uint64_t* x, uint64_t* sm, uint32_t tid) {
  constexpr int E = NttShape<LOGN>::E;
  const uint32_t base = swz8(inv_index<LOGN, U0, K>(tid, 0, 0));
#pragma unroll
  for (int e = 0; e < E; e++) x[e] = sm_at(sm, base ^ swz8(inv_index<LOGN, U0, K>(0, e >> K, e & ((1 << K) - 1))));
}

// Size of the first inverse round: the remainder, so that later rounds are
// full and the last round stores coalesced.
template <int LOGN>
struct InvFirst {
  static constexpr int LOGE = NttShape<LOGN>::LOGE;
  static constexpr int K = (LOGN % LOGE) ? (LOGN % LOGE) : LOGE;
};

template <int LOGN, int U0, int K>
__device__ __forceinline__ void inv_rounds(uint64_t* x, uint64_t* sm, uint32_t tid, const DevPrime& pr,
                                           uint32_t n_total, uint32_t s1, uint32_t beta) {
  constexpr int LOGE = NttShape<LOGN>::LOGE;
  inv_round<LOGN, U0, K>(x, tid, pr, n_total, s1, beta);
  if constexpr (U0 + K < LOGN) {
    constexpr int K2 = (LOGN - U0 - K) < LOGE ? (LOGN - U0 - K) : LOGE;
    __syncthreads();
    inv_to_smem<LOGN, U0, K>(x, sm, tid);
    __syncthreads();
    inv_from_smem<LOGN, U0 + K, K2>(x, sm, tid);
    inv_rounds<LOGN, U0 + K, K2>(x, sm, tid, pr, n_total, s1, beta);
  }
}

// Inverse NTT of blocks of 2^LOGN elements (all GS stages with l < 2^LOGN).
// With g.s1 = 0 this is the whole `backward`, including the N^-1 scaling
// (FINAL). With g.s1 > 0 the remaining stages run in ntt_inv_top.
template <int LOGN, bool FINAL, class Src, class Dst>
__global__ void __launch_bounds__(NttShape<LOGN>::T, NttShape<LOGN>::MIN_BLOCKS) k_ntt_inv(NttGeom g, Src src, Dst dst) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  constexpr int K0 = InvFirst<LOGN>::K;
  extern __shared__ uint64_t sm[];
  const uint32_t tid = threadIdx.x;
  const NttJob jb = decode_job(g);
  const DevPrime pr = g.primes[jb.limb];
  const uint32_t base = jb.beta << LOGN;
  prefetch_next<LOGN, T>(g, src, tid);
  uint64_t x[E];
  // Coalesced loads, then regroup through shared memory for the first round.
  // (Staging a single row the same way measured slower: the extra shared-
  // memory round trip costs more than the load latency it hides.)
  const uint32_t sb = swz8(tid);
  if constexpr (src_is_staged<Src>(0)) {
    src.template stage<LOGN, T, E>(jb, pr, base, sm, tid, x);
#pragma unroll
    for (int e = 0; e < E; e++) sm_at(sm, sb ^ swz8(e * T)) = x[e];
  } else {
#pragma unroll
    for (int e = 0; e < E; e++) {
      const uint32_t i = tid + e * T;
      sm_at(sm, sb ^ swz8(e * T)) = src(jb, pr, base + i);
    }
  }
  __syncthreads();
  inv_from_smem<LOGN, 0, K0>(x, sm, tid);
  inv_rounds<LOGN, 0, K0>(x, sm, tid, pr, 1u << (LOGN + g.s1), g.s1, jb.beta);
  // The last round holds elements tid + e*T (b = tid, c = 0): coalesced stores.
#pragma unroll
  for (int e = 0; e < E; e++) {
    uint64_t v = x[e];
    if (FINAL) v = inv_final_scale(g, pr, v);
    dst(jb, pr, base + tid + e * T, v);
  }
}

// ---------------------------------------------------------------------------
// Small transforms (N <= 2^11, used by small parameter sets and tests): one
// CTA per limb, radix-2 stages in shared memory, the size a runtime value.
// Same butterflies and twiddle indices as above, so the same outputs.

template <bool REDUCE, class Src, class Dst>
__global__ void __launch_bounds__(1024) k_ntt_fwd_small(NttGeom g, uint32_t logn, Src src, Dst dst) {
  extern __shared__ uint64_t sm[];
  const uint32_t n = 1u << logn, tid = threadIdx.x, nt = blockDim.x;
  const NttJob jb = decode_job(g);
  const DevPrime pr = g.primes[jb.limb];
  for (uint32_t i = tid; i < n; i += nt) sm[i] = src(jb, pr, i);
  __syncthreads();
  for (uint32_t s = 0; s < logn; s++) {
    const uint32_t l = n >> (s + 1);
    for (uint32_t b = tid; b < n / 2; b += nt) {
      const uint32_t chunk = b / l, j = chunk * 2 * l + (b % l);
      const ulonglong2 w = __ldg(pr.tw + (1u << s) + chunk);
      uint64_t x = sm[j], y = sm[j + l];
      fwd_bfly(x, y, w.x, w.y, pr.p, pr.p2);
      sm[j] = x;
      sm[j + l] = y;
    }
    __syncthreads();
  }
  for (uint32_t i = tid; i < n; i += nt) dst(jb, pr, i, REDUCE ? reduce4(sm[i], pr.p, pr.p2) : sm[i]);
}

template <class Src, class Dst>
__global__ void __launch_bounds__(1024) k_ntt_inv_small(NttGeom g, uint32_t logn, Src src, Dst dst) {
  extern __shared__ uint64_t sm[];
  const uint32_t n = 1u << logn, tid = threadIdx.x, nt = blockDim.x;
  const NttJob jb = decode_job(g);
  const DevPrime pr = g.primes[jb.limb];
  for (uint32_t i = tid; i < n; i += nt) sm[i] = src(jb, pr, i);
  __syncthreads();
  for (uint32_t l = 1; l < n; l <<= 1) {
    const uint32_t m = n / (2 * l);
    for (uint32_t b = tid; b < n / 2; b += nt) {
      const uint32_t chunk = b / l, j = chunk * 2 * l + (b % l);
      const ulonglong2 z = __ldg(pr.itw + (n - 2 * m + chunk));
      uint64_t x = sm[j], y = sm[j + l];
      inv_bfly(x, y, z.x, z.y, pr.p, pr.p2);
      sm[j] = x;
      sm[j + l] = y;
    }
    __syncthreads();
  }
  for (uint32_t i = tid; i < n; i += nt) dst(jb, pr, i, inv_final_scale(g, pr, sm[i]));
}

// ---------------------------------------------------------------------------
// Strided passes for N = 2^(LOGB + S1) with 1 <= S1 <= 4: the first S1
// forward stages / the last S1 inverse stages, on groups of 2^S1 elements
// b + t * 2^LOGB. One thread per group.

// The first S1 forward stages of a transform on the 2^S1 elements
// x[t] = element b + t * N / 2^S1 of one limb (inputs below 4p, outputs lazy
// in [0, 4p)): what the strided forward pass does per thread, also applied
// by producers that write the block pass's input directly (the RNS scaler of
// the multiplication).
template <int S1>
__device__ __forceinline__ void fwd_top_stages(uint64_t* x, const DevPrime& pr) {
#pragma unroll
  for (int s = 0; s < S1; s++) {
    const int half = 1 << (S1 - 1 - s);
#pragma unroll
    for (int k = 0; k < (1 << s); k++) {
      const ulonglong2 wp = __ldg(pr.tw + (1u << s) + k);
      const uint64_t w = wp.x, ws = wp.y;
#pragma unroll
      for (int u = 0; u < half; u++) {
        const int t = (k << (S1 - s)) + u;
        fwd_bfly(x[t], x[t + half], w, ws, pr.p, pr.p2);
      }
    }
  }
}

template <int S1, class Src, class Dst>
__global__ void __launch_bounds__(256) k_ntt_fwd_top(NttGeom g, uint32_t logb, uint32_t groups_per_limb,
                                                     uint64_t total, Src src, Dst dst) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t b = (uint32_t)gid & (groups_per_limb - 1);  // groups_per_limb = 2^logb
  const NttJob jb = unit_job(g, row_of(gid, logb));
  const DevPrime pr = g.primes[jb.limb];
  uint64_t x[1 << S1];
#pragma unroll
  for (int t = 0; t < (1 << S1); t++) x[t] = src(jb, pr, b + ((uint32_t)t << logb));
  fwd_top_stages<S1>(x, pr);
#pragma unroll
  for (int t = 0; t < (1 << S1); t++) dst(jb, pr, b + ((uint32_t)t << logb), x[t]);
}

// The last S1 inverse stages of a transform of n_total residues and its
// final scale (N^-1, or N^-1 * 2^64 when `mont`), on the 2^S1 elements
// x[t] = element b + t * n_total / 2^S1 of one limb: what the strided inverse
// pass does per thread, also applied by consumers that read the block pass's
// output directly (the RNS scaler of the multiplication).
template <int S1>
__device__ __forceinline__ void inv_top_stages(uint64_t* x, const DevPrime& pr, uint32_t n_total, bool mont) {
#pragma unroll
  for (int r = 0; r < S1 - 1; r++) {
    const int span = 1 << r;
    const uint32_t m = 1u << (S1 - 1 - r);  // chunks at this stage
#pragma unroll
    for (int k = 0; k < (1 << (S1 - 1 - r)); k++) {
      const ulonglong2 zp = __ldg(pr.itw + (n_total - 2 * m + k));
      const uint64_t z = zp.x, zs = zp.y;
#pragma unroll
      for (int u = 0; u < span; u++) {
        const int t = (k << (r + 1)) + u;
        inv_bfly(x[t], x[t + span], z, zs, pr.p, pr.p2);
      }
    }
  }
  // The last stage (one chunk, twiddle zetas_inv[N - 2]) with the final
  // scale folded into its products.
  const uint64_t s = mont ? pr.ninv_mont : pr.ninv, s_shoup = mont ? pr.ninv_mont_shoup : pr.ninv_shoup;
  const uint64_t zs = mont ? pr.zlast_ninv_mont : pr.zlast_ninv;
  const uint64_t zs_shoup = mont ? pr.zlast_ninv_mont_shoup : pr.zlast_ninv_shoup;
  constexpr int kHalf = 1 << (S1 - 1);
#pragma unroll
  for (int u = 0; u < kHalf; u++) inv_bfly_final(x[u], x[u + kHalf], zs, zs_shoup, s, s_shoup, pr.p, pr.p2);
}

template <int S1, class Src, class Dst>
__global__ void __launch_bounds__(256) k_ntt_inv_top(NttGeom g, uint32_t logb, uint32_t groups_per_limb,
                                                     uint64_t total, Src src, Dst dst) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t b = (uint32_t)gid & (groups_per_limb - 1);  // groups_per_limb = 2^logb
  const NttJob jb = unit_job(g, row_of(gid, logb));
  const DevPrime pr = g.primes[jb.limb];
  uint64_t x[1 << S1];
#pragma unroll
  for (int t = 0; t < (1 << S1); t++) x[t] = src(jb, pr, b + ((uint32_t)t << logb));
  inv_top_stages<S1>(x, pr, 1u << (logb + S1), g.mont != 0);
#pragma unroll
  for (int t = 0; t < (1 << S1); t++) dst(jb, pr, b + ((uint32_t)t << logb), x[t]);
}

// ---------------------------------------------------------------------------
// Single-pass transforms of 2^(12 + s1) residues (s1 = 1..4) on a cluster of
// 2^s1 CTAs: CTA r of the cluster holds block r (2^12 residues) in its shared
// memory, and the strided stages (the first s1 forward / last s1 inverse)
// exchange through distributed shared memory instead of a second pass over
// HBM. Every thread of every CTA reaches both cluster barriers, which are
// hardware barriers among co-scheduled CTAs.

// Shared::cluster address of word offset `off8` (bytes) of CTA `rank`'s
// dynamic shared memory.
__device__ __forceinline__ uint32_t cluster_addr(uint64_t* sm, uint32_t rank, uint32_t off8) {
  uint32_t out;
  const uint32_t local = (uint32_t)__cvta_generic_to_shared(sm) + off8;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(local), "r"(rank));
  return out;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, uint64_t v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_cluster(uint32_t addr) {
  uint64_t v;
  asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(addr) : "memory");
  return v;
}
// All threads of all CTAs of the cluster; orders the shared-memory writes
// before it with the reads after it, across the cluster.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// The two halves of a barrier that only establishes that every CTA of the
// cluster has started (before the first write into a peer's shared memory).
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }

// Forward phase 1: the first S1 stages on the groups b + t 2^LOGB (t < 2^S1)
// with b in this CTA's share of [0, 2^LOGB); element b + t 2^LOGB lands at
// local index b of CTA t.
template <int LOGB, int S1, class Src>
__device__ __forceinline__ void fwd_cluster_top(const Src& src, const NttJob& jb, const DevPrime& pr, uint64_t* sm,
                                                uint32_t tid, uint32_t rank) {
  constexpr int E = NttShape<LOGB>::E, T = NttShape<LOGB>::T, C = 1 << S1, GPT = E / C;
  constexpr uint32_t NB = 1u << LOGB;
  static_assert(GPT >= 1, "cluster larger than the residues per thread");
  const uint32_t b0 = rank * (NB / C) + tid;  // bits of rank, tid and q * T are disjoint
  uint64_t x[E];
#pragma unroll
  for (int q = 0; q < GPT; q++)
#pragma unroll
    for (int t = 0; t < C; t++) x[q * C + t] = src(jb, pr, b0 + q * T + t * NB);
#pragma unroll
  for (int q = 0; q < GPT; q++) fwd_top_stages<S1>(x + q * C, pr);
  const uint32_t sb = swz8(b0);
  cluster_wait();  // every peer has started (arrival at kernel entry)
#pragma unroll
  for (int t = 0; t < C; t++) {
    const uint32_t peer = cluster_addr(sm, t, 0);
#pragma unroll
    for (int q = 0; q < GPT; q++) st_cluster(peer + (sb ^ swz8(q * T)), x[q * C + t]);
  }
}

template <int LOGN, bool REDUCE, class Src, class Dst>
__global__ void __launch_bounds__(NttShape<LOGN>::T, NttShape<LOGN>::MIN_BLOCKS)
    k_ntt_fwd_cl(NttGeom g, Src src, Dst dst) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  extern __shared__ uint64_t sm[];
  const uint32_t tid = threadIdx.x;
  cluster_arrive_relaxed();
  const NttJob jb = decode_job(g);  // beta = the CTA's rank in its cluster
  const DevPrime pr = g.primes[jb.limb];
  switch (g.s1) {
    case 1: fwd_cluster_top<LOGN, 1>(src, jb, pr, sm, tid, jb.beta); break;
    case 2: fwd_cluster_top<LOGN, 2>(src, jb, pr, sm, tid, jb.beta); break;
    case 3: fwd_cluster_top<LOGN, 3>(src, jb, pr, sm, tid, jb.beta); break;
    default: fwd_cluster_top<LOGN, 4>(src, jb, pr, sm, tid, jb.beta); break;
  }
  cluster_sync();
  uint64_t x[E];
  const uint32_t sb = swz8(tid);
#pragma unroll
  for (int e = 0; e < E; e++) x[e] = sm_at(sm, sb ^ swz8(e * T));
  fwd_rounds<LOGN, 0>(x, sm, tid, pr, (1u << g.s1) + jb.beta);
  const uint32_t base = jb.beta << LOGN;
#pragma unroll
  for (int e = 0; e < E; e++) {
    uint64_t v = sm_at(sm, sb ^ swz8(e * T));
    if (REDUCE) v = reduce4(v, pr.p, pr.p2);
    dst(jb, pr, base + tid + e * T, v);
  }
}

// Inverse phase 2: the last S1 stages (and the final scale) on the groups of
// this CTA's share, read from the cluster's blocks.
template <int LOGB, int S1, class Dst>
__device__ __forceinline__ void inv_cluster_top(const NttGeom& g, const Dst& dst, const NttJob& jb,
                                                const DevPrime& pr, uint64_t* sm, uint32_t tid, uint32_t rank) {
  constexpr int E = NttShape<LOGB>::E, T = NttShape<LOGB>::T, C = 1 << S1, GPT = E / C;
  constexpr uint32_t NB = 1u << LOGB;
  const uint32_t b0 = rank * (NB / C) + tid;
  const uint32_t sb = swz8(b0);
  uint64_t x[E];
#pragma unroll
  for (int t = 0; t < C; t++) {
    const uint32_t peer = cluster_addr(sm, t, 0);
#pragma unroll
    for (int q = 0; q < GPT; q++) x[q * C + t] = ld_cluster(peer + (sb ^ swz8(q * T)));
  }
#pragma unroll
  for (int q = 0; q < GPT; q++) inv_top_stages<S1>(x + q * C, pr, NB << S1, g.mont != 0);
#pragma unroll
  for (int q = 0; q < GPT; q++)
#pragma unroll
    for (int t = 0; t < C; t++) dst(jb, pr, b0 + q * T + t * NB, x[q * C + t]);
}

template <int LOGN, class Src, class Dst>
__global__ void __launch_bounds__(NttShape<LOGN>::T, NttShape<LOGN>::MIN_BLOCKS)
    k_ntt_inv_cl(NttGeom g, Src src, Dst dst) {
  constexpr int E = NttShape<LOGN>::E;
  constexpr int T = NttShape<LOGN>::T;
  constexpr int K0 = InvFirst<LOGN>::K;
  extern __shared__ uint64_t sm[];
  const uint32_t tid = threadIdx.x;
  const NttJob jb = decode_job(g);
  const DevPrime pr = g.primes[jb.limb];
  const uint32_t base = jb.beta << LOGN;
  uint64_t x[E];
  const uint32_t sb = swz8(tid);
  if constexpr (src_is_staged<Src>(0)) {
    src.template stage<LOGN, T, E>(jb, pr, base, sm, tid, x);
#pragma unroll
    for (int e = 0; e < E; e++) sm_at(sm, sb ^ swz8(e * T)) = x[e];
  } else {
#pragma unroll
    for (int e = 0; e < E; e++) sm_at(sm, sb ^ swz8(e * T)) = src(jb, pr, base + tid + e * T);
  }
  __syncthreads();
  inv_from_smem<LOGN, 0, K0>(x, sm, tid);
  inv_rounds<LOGN, 0, K0>(x, sm, tid, pr, 1u << (LOGN + g.s1), g.s1, jb.beta);
  // Every thread has read its last exchange: the block's results go to
  // shared memory for the cluster.
  __syncthreads();
#pragma unroll
  for (int e = 0; e < E; e++) sm_at(sm, sb ^ swz8(e * T)) = x[e];
  cluster_sync();
  switch (g.s1) {
    case 1: inv_cluster_top<LOGN, 1>(g, dst, jb, pr, sm, tid, jb.beta); break;
    case 2: inv_cluster_top<LOGN, 2>(g, dst, jb, pr, sm, tid, jb.beta); break;
    case 3: inv_cluster_top<LOGN, 3>(g, dst, jb, pr, sm, tid, jb.beta); break;
    default: inv_cluster_top<LOGN, 4>(g, dst, jb, pr, sm, tid, jb.beta); break;
  }
  // No CTA leaves while another may still read its shared memory.
  cluster_sync();
}

// ---------------------------------------------------------------------------
// Basic source / destination functors.

struct SrcPoly {
  PolyRef r;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return r.at(j.poly, j.limb)[i];
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const { prefetch_l2(r.at(j.poly, j.limb) + i); }
};

// Destinations also provide `reload`, which the two-pass sizes use to read
// back the intermediate values the first pass stored.
struct DstPoly {
  PolyRef r;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    r.at(j.poly, j.limb)[i] = v;
  }
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const { return r.at(j.poly, j.limb)[i]; }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const { prefetch_l2(r.at(j.poly, j.limb) + i); }
};

template <class Dst>
struct SrcReload {
  Dst d;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return d.reload(j, i);
  }
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const { src_prefetch(d, j, i, 0); }
};

// ---------------------------------------------------------------------------
// Launch helpers.

template <int LOGN>
inline size_t ntt_smem_bytes() {
  return sizeof(uint64_t) << LOGN;
}

// Opts a kernel into more than 48 KB of dynamic shared memory (once per
// kernel; `done` is a per-instantiation flag).
template <class K>
inline void set_smem(K kernel, size_t bytes, bool* done) {
  if (bytes > 48 * 1024 && !*done) {
    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
               "cudaFuncSetAttribute");
    *done = true;
  }
}

// CTAs resident on the whole GPU at once for a kernel (the distance to the
// CTA that takes a finished one's place), computed once per kernel.
template <class K>
inline uint32_t resident_ctas(K kernel, int threads, size_t smem, uint32_t* cache) {
  if (*cache == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem), "occupancy");
    *cache = (uint32_t)std::max(1, sms * std::max(per_sm, 1));
  }
  return *cache;
}

template <int LOGN, bool REDUCE, class Src, class Dst>
void launch_fwd_block(NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  auto kern = k_ntt_fwd<LOGN, REDUCE, Src, Dst>;
  const size_t smem = ntt_smem_bytes<LOGN>();
  static bool done = false;
  set_smem(kern, smem, &done);
  static uint32_t resident = 0;
  g.pf_stride = ntt_prefetch_enabled() ? resident_ctas(kern, NttShape<LOGN>::T, smem, &resident) : 0;
  const uint64_t blocks = polys * g.limbs << g.s1;
  kern<<<(unsigned)blocks, NttShape<LOGN>::T, smem, st>>>(g, src, dst);
  after_launch("k_ntt_fwd");
}

template <int LOGN, bool FINAL, class Src, class Dst>
void launch_inv_block(NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  auto kern = k_ntt_inv<LOGN, FINAL, Src, Dst>;
  const size_t smem = ntt_smem_bytes<LOGN>();
  static bool done = false;
  set_smem(kern, smem, &done);
  static uint32_t resident = 0;
  g.pf_stride = ntt_prefetch_enabled() ? resident_ctas(kern, NttShape<LOGN>::T, smem, &resident) : 0;
  const uint64_t blocks = polys * g.limbs << g.s1;
  kern<<<(unsigned)blocks, NttShape<LOGN>::T, smem, st>>>(g, src, dst);
  after_launch("k_ntt_inv");
}

// Launch of a kernel on clusters of `csize` CTAs along x.
template <class K, class... Args>
void launch_cluster(K kern, uint64_t blocks, unsigned threads, size_t smem, unsigned csize, cudaStream_t st,
                    Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks, 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  check_cuda(cudaLaunchKernelEx(&cfg, kern, args...), "cudaLaunchKernelEx");
}

// Whether clusters of 2^s1 CTAs of `kern` fit on the GPU (state per s1:
// 0 unknown, 1 yes, -1 no; computed once). 16-CTA clusters need the
// non-portable size opt-in.
template <class K>
bool cluster_fits(K kern, uint32_t s1, unsigned threads, size_t smem, int* state) {
  if (s1 < 1 || s1 > 4) return false;
  if (state[s1] == 0) {
    int n = 0;
    bool ok = true;
    if (s1 == 4) ok = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
    if (ok) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(1u << s1, 1, 1);
      cfg.blockDim = dim3(threads, 1, 1);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 1u << s1;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      ok = cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n > 0;
    }
    if (!ok) (void)cudaGetLastError();
    state[s1] = ok ? 1 : -1;
  }
  return state[s1] > 0;
}

// Single-pass cluster transforms of 2^(LOGN + s1) residues; false (nothing
// launched) when the GPU cannot run the cluster size.
template <int LOGN, bool REDUCE, class Src, class Dst>
bool launch_fwd_cluster(NttGeom g, uint32_t s1, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  auto kern = k_ntt_fwd_cl<LOGN, REDUCE, Src, Dst>;
  const size_t smem = ntt_smem_bytes<LOGN>();
  static bool done = false;
  set_smem(kern, smem, &done);
  static int fits[5] = {0, 0, 0, 0, 0};
  if (!cluster_fits(kern, s1, NttShape<LOGN>::T, smem, fits)) return false;
  g.s1 = s1;
  g.pf_stride = 0;
  launch_cluster(kern, polys * g.limbs << s1, NttShape<LOGN>::T, smem, 1u << s1, st, g, src, dst);
  after_launch("k_ntt_fwd_cl");
  return true;
}

template <int LOGN, class Src, class Dst>
bool launch_inv_cluster(NttGeom g, uint32_t s1, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  auto kern = k_ntt_inv_cl<LOGN, Src, Dst>;
  const size_t smem = ntt_smem_bytes<LOGN>();
  static bool done = false;
  set_smem(kern, smem, &done);
  static int fits[5] = {0, 0, 0, 0, 0};
  if (!cluster_fits(kern, s1, NttShape<LOGN>::T, smem, fits)) return false;
  g.s1 = s1;
  g.pf_stride = 0;
  launch_cluster(kern, polys * g.limbs << s1, NttShape<LOGN>::T, smem, 1u << s1, st, g, src, dst);
  after_launch("k_ntt_inv_cl");
  return true;
}

// Dispatch over log2(N) for a single-pass transform (3 <= logn <= 14).
constexpr uint32_t kMinUnrolledLogN = 12;

template <bool REDUCE, class Src, class Dst>
void ntt_fwd_single(uint32_t logn, NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  switch (logn) {
    case 12: launch_fwd_block<12, REDUCE>(g, polys, src, dst, st); break;
    case 13: launch_fwd_block<13, REDUCE>(g, polys, src, dst, st); break;
    case 14: launch_fwd_block<14, REDUCE>(g, polys, src, dst, st); break;
    default: {
      if (logn < 3 || logn > 11) throw Error(12, "unsupported NTT size");
      const uint32_t threads = logn >= 11 ? 1024 : (1u << (logn - 1));
      const uint64_t blocks = polys * g.limbs;
      k_ntt_fwd_small<REDUCE><<<(unsigned)blocks, threads, (sizeof(uint64_t) << logn), st>>>(g, logn, src, dst);
      after_launch("k_ntt_fwd_small");
    }
  }
}

template <bool FINAL, class Src, class Dst>
void ntt_inv_single(uint32_t logn, NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  switch (logn) {
    case 12: launch_inv_block<12, FINAL>(g, polys, src, dst, st); break;
    case 13: launch_inv_block<13, FINAL>(g, polys, src, dst, st); break;
    case 14: launch_inv_block<14, FINAL>(g, polys, src, dst, st); break;
    default: {
      if (logn < 3 || logn > 11 || !FINAL) throw Error(12, "unsupported NTT size");
      const uint32_t threads = logn >= 11 ? 1024 : (1u << (logn - 1));
      const uint64_t blocks = polys * g.limbs;
      k_ntt_inv_small<<<(unsigned)blocks, threads, (sizeof(uint64_t) << logn), st>>>(g, logn, src, dst);
      after_launch("k_ntt_inv_small");
    }
  }
}

// Two-pass transforms: a strided pass runs the first (forward) or last
// (inverse) s1 stages on groups of 2^s1 elements b + t * 2^bl, and the block
// kernel runs the other bl stages on 2^s1 blocks of 2^bl elements.
template <class Src, class Dst>
void launch_fwd_top(uint32_t s1, NttGeom g, uint32_t bl, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  const uint32_t groups = 1u << bl;
  const uint64_t threads = polys * g.limbs * groups;
  const unsigned blocks = (unsigned)((threads + 255) / 256);
  g.s1 = 0;
  switch (s1) {
    case 1: k_ntt_fwd_top<1><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 2: k_ntt_fwd_top<2><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 3: k_ntt_fwd_top<3><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 4: k_ntt_fwd_top<4><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    default: throw Error(12, "unsupported NTT plan");
  }
  after_launch("k_ntt_fwd_top");
}

template <class Src, class Dst>
void launch_inv_top(uint32_t s1, NttGeom g, uint32_t bl, uint64_t polys, Src src, Dst dst, cudaStream_t st) {
  const uint32_t groups = 1u << bl;
  const uint64_t threads = polys * g.limbs * groups;
  const unsigned blocks = (unsigned)((threads + 255) / 256);
  g.s1 = 0;
  switch (s1) {
    case 1: k_ntt_inv_top<1><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 2: k_ntt_inv_top<2><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 3: k_ntt_inv_top<3><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    case 4: k_ntt_inv_top<4><<<blocks, 256, 0, st>>>(g, bl, groups, threads, src, dst); break;
    default: throw Error(12, "unsupported NTT plan");
  }
  after_launch("k_ntt_inv_top");
}

// Full forward NTT, any 3 <= logn <= 16, following the plan of
// ntt_block_logn(logn): single pass, or a strided pass that reads `src` and
// writes its lazy output to `dst`, then the block pass that reads it back.
// `bl` selects the plan explicitly (0 = the process-wide plan of logn).
template <bool REDUCE, class Src, class Dst>
void ntt_forward_any(uint32_t logn, NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st,
                     uint32_t bl = 0) {
  if (bl == 0) bl = ntt_block_logn(logn);
  if (bl >= logn || logn < 13) {
    g.s1 = 0;
    ntt_fwd_single<REDUCE>(logn, g, polys, src, dst, st);
    return;
  }
  const uint32_t s1 = logn - bl;
  if (bl == 12 && ntt_cluster_enabled(logn) && launch_fwd_cluster<12, REDUCE>(g, s1, polys, src, dst, st)) return;
  launch_fwd_top(s1, g, bl, polys, src, dst, st);
  g.s1 = s1;
  switch (bl) {
    case 12: launch_fwd_block<12, REDUCE>(g, polys, SrcReload<Dst>{dst}, dst, st); break;
    case 13: launch_fwd_block<13, REDUCE>(g, polys, SrcReload<Dst>{dst}, dst, st); break;
    case 14: launch_fwd_block<14, REDUCE>(g, polys, SrcReload<Dst>{dst}, dst, st); break;
    default: throw Error(12, "unsupported NTT plan");
  }
}

// The block pass of a two-pass forward NTT of `dst` in place, for data whose
// strided first logn - bl stages a producer already applied
// (fwd_top_stages). Requires a two-pass plan.
// `from` (a destination functor) names where the producer left that data
// when it is not `dst` itself.
template <bool REDUCE, class From, class Dst>
void ntt_forward_after_top(uint32_t logn, NttGeom g, uint64_t polys, From from, Dst dst, cudaStream_t st,
                           uint32_t bl = 0) {
  if (bl == 0) bl = ntt_block_logn(logn);
  if (bl >= logn || logn < 13) throw Error(12, "the forward NTT plan has no strided stages");
  g.s1 = logn - bl;
  switch (bl) {
    case 12: launch_fwd_block<12, REDUCE>(g, polys, SrcReload<From>{from}, dst, st); break;
    case 13: launch_fwd_block<13, REDUCE>(g, polys, SrcReload<From>{from}, dst, st); break;
    case 14: launch_fwd_block<14, REDUCE>(g, polys, SrcReload<From>{from}, dst, st); break;
    default: throw Error(12, "unsupported NTT plan");
  }
}

template <bool REDUCE, class Dst>
void ntt_forward_after_top(uint32_t logn, NttGeom g, uint64_t polys, Dst dst, cudaStream_t st, uint32_t bl = 0) {
  ntt_forward_after_top<REDUCE>(logn, g, polys, dst, dst, st, bl);
}

// Full inverse NTT, any 3 <= logn <= 16: single pass, or the block pass into
// `dst` followed by the strided pass in place.
template <class Src, class Dst>
void ntt_inverse_any(uint32_t logn, NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st,
                     uint32_t bl = 0) {
  g.mont = src_is_montgomery<Src>(0) ? 1u : 0u;
  if (bl == 0) bl = ntt_block_logn(logn);
  if (bl >= logn || logn < 13) {
    g.s1 = 0;
    ntt_inv_single<true>(logn, g, polys, src, dst, st);
    return;
  }
  const uint32_t s1 = logn - bl;
  if (bl == 12 && ntt_cluster_enabled(logn) && launch_inv_cluster<12>(g, s1, polys, src, dst, st)) return;
  g.s1 = s1;
  switch (bl) {
    case 12: launch_inv_block<12, false>(g, polys, src, dst, st); break;
    case 13: launch_inv_block<13, false>(g, polys, src, dst, st); break;
    case 14: launch_inv_block<14, false>(g, polys, src, dst, st); break;
    default: throw Error(12, "unsupported NTT plan");
  }
  launch_inv_top(s1, g, bl, polys, SrcReload<Dst>{dst}, dst, st);
}

// The inverse NTT up to its strided last stages: with a two-pass plan only the
// block pass runs, and the caller's consumer applies the remaining stages
// (inv_top_stages) as it reads `dst`; returns their number (0: the transform
// ran whole, single pass).
template <class Src, class Dst>
uint32_t ntt_inverse_blocks(uint32_t logn, NttGeom g, uint64_t polys, Src src, Dst dst, cudaStream_t st,
                            uint32_t bl = 0) {
  g.mont = src_is_montgomery<Src>(0) ? 1u : 0u;
  if (bl == 0) bl = ntt_block_logn(logn);
  if (bl >= logn || logn < 13) {
    ntt_inverse_any(logn, g, polys, src, dst, st, bl);
    return 0;
  }
  const uint32_t s1 = logn - bl;
  g.s1 = s1;
  switch (bl) {
    case 12: launch_inv_block<12, false>(g, polys, src, dst, st); break;
    case 13: launch_inv_block<13, false>(g, polys, src, dst, st); break;
    case 14: launch_inv_block<14, false>(g, polys, src, dst, st); break;
    default: throw Error(12, "unsupported NTT plan");
  }
  return s1;
}

}  // namespace
}  // namespace fheg
