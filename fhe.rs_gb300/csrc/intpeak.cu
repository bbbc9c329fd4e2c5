// Integer-throughput probes: the ceilings the NTT and RNS kernels are
// measured against. Every kernel runs 8 independent dependency chains per
// thread on register-resident values (no memory traffic but one store per
// thread at the end, so the work stays live), which makes each launch bound by
// the issue rate of the probed operation alone.

#include <cuda_runtime.h>
#include <stdint.h>

#include "abi_call.hpp"
#include "common.cuh"
#include "fheg.h"
#include "lib.hpp"

namespace {

constexpr int kChains = 8;

// 32-bit multiply-add, low half (the IMAD of every residue product).
__global__ void k_probe_mad_lo(uint32_t a, uint32_t b, uint32_t iters, uint64_t* sink) {
  uint32_t acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) acc[k] = threadIdx.x + k;
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(acc[k]) : "r"(a), "r"(b));
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += acc[k];
  sink[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// 32 x 32 -> 64-bit multiply-add (the wide partial products).
__global__ void k_probe_mad_wide(uint32_t b, uint32_t iters, uint64_t* sink) {
  uint64_t acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) acc[k] = threadIdx.x + k;
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++)
      asm volatile("{\n\t.reg .u32 lo, hi;\n\tmov.b64 {lo, hi}, %0;\n\tmad.wide.u32 %0, lo, %1, %0;\n\t}"
                   : "+l"(acc[k])
                   : "r"(b));
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += acc[k];
  sink[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// High half of a 32 x 32-bit product, with an addend.
__global__ void k_probe_mad_hi(uint32_t b, uint32_t c, uint32_t iters, uint64_t* sink) {
  uint32_t acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) acc[k] = threadIdx.x * 977u + k;
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) asm volatile("mad.hi.u32 %0, %0, %1, %2;" : "+r"(acc[k]) : "r"(b), "r"(c));
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += acc[k];
  sink[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Three-input 32-bit addition (the carries and lazy-range arithmetic).
__global__ void k_probe_add3(uint32_t b, uint32_t c, uint32_t iters, uint64_t* sink) {
  uint32_t acc[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) acc[k] = threadIdx.x + k;
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++)
      asm volatile("{\n\t.reg .u32 t;\n\tadd.u32 t, %0, %1;\n\tadd.u32 %0, t, %2;\n\t}" : "+r"(acc[k]) : "r"(b), "r"(c));
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += acc[k];
  sink[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The NTT's butterflies (ntt.cuh / common.cuh) on register-resident values,
// with one twiddle and its Shoup companion: Harvey forward (lazy [0, 4p)) or
// Gentleman-Sande inverse ([0, 2p)).
template <bool FWD>
__global__ void k_probe_bfly(uint64_t w, uint64_t ws, uint64_t p, uint32_t iters, uint64_t* sink) {
  uint64_t x[kChains], y[kChains];
  const uint64_t p2 = 2 * p;
#pragma unroll
  for (int k = 0; k < kChains; k++) {
    x[k] = (threadIdx.x * 7919ull + k) % p;
    y[k] = (threadIdx.x * 104729ull + 3 * k + 1) % p;
  }
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) {
      if (FWD) fheg::fwd_bfly(x[k], y[k], w, ws, p, p2);
      else fheg::inv_bfly(x[k], y[k], w, ws, p, p2);
    }
  }
  uint64_t s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k] ^ y[k];
  sink[(uint64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

FHEG_API int fheg_intpeak(int kind, size_t blocks, uint32_t iters, uint64_t* d_sink, void* stream, double* ops) {
  using namespace fheg;
  return abi_call([&] {
    abi_need(d_sink && ops && blocks > 0 && blocks <= (1u << 20), "invalid probe launch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned g = (unsigned)blocks;
    // A 62-bit NTT prime and a twiddle below it, with its Shoup companion.
    const uint64_t p = 4611686018427322369ull, w = 1234567890123456789ull % p;
    const uint64_t ws = (uint64_t)(((unsigned __int128)w << 64) / p);
    switch (kind) {
      case 0: k_probe_mad_lo<<<g, 256, 0, st>>>(0x9E3779B9u, 12345u, iters, d_sink); break;
      case 1: k_probe_mad_wide<<<g, 256, 0, st>>>(0x9E3779B9u, iters, d_sink); break;
      case 2: k_probe_mad_hi<<<g, 256, 0, st>>>(0x9E3779B9u, 12345u, iters, d_sink); break;
      case 3: k_probe_add3<<<g, 256, 0, st>>>(0x9E3779B9u, 12345u, iters, d_sink); break;
      case 4: k_probe_bfly<true><<<g, 256, 0, st>>>(w, ws, p, iters, d_sink); break;
      case 5: k_probe_bfly<false><<<g, 256, 0, st>>>(w, ws, p, iters, d_sink); break;
      default: throw Error(FHEG_ERR_INVALID_ARGUMENT, "unknown probe kind");
    }
    after_launch("k_probe");
    // Operations performed: one per chain and iteration (kind 3 counts each
    // of its two additions).
    *ops = (double)blocks * 256.0 * (double)iters * kChains * (kind == 3 ? 2.0 : 1.0);
  });
}
