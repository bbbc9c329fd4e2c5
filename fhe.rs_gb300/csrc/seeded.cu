// Polynomials expanded from 32-byte seeds on the device:
// Poly::random_from_seed (fhe-math/src/rq/mod.rs:239-257), which fresh
// seeded ciphertexts use for c1 (fhe/src/bfv/ciphertext.rs:220-237) and
// seeded key-switching keys for every c1[i] (key_switching_key.rs:108-123,
// 383-406).
//
// The reference hashes the seed with SHA-256 (sha2 0.10.9), keys a ChaCha8
// generator with the digest (rand_chacha 0.9.0: 64-bit block counter, 64-bit
// stream id, both starting at zero) and fills each limb in turn with N
// samples of Uniform[0, q_j) (rand 0.9.2 UniformInt<u64>: the high word of the
// 128-bit product draw * q_j, the draw rejected when the low word is below
// (2^64 - q_j) mod q_j). Draw k is keystream words 2k (low) and 2k+1 (high).
//
// Device plan: one thread per seed computes the digest; then one thread per
// ChaCha block (8 draws) computes its outputs at the positions they take when
// no draw is rejected, and flags the polynomial if one of its draws would be
// rejected. For moduli close to 2^62 that happens with probability ~2^-46 per
// draw; a flagged polynomial is recomputed by one warp that walks the draws
// in order (32 at a time, ballot + prefix count), which is exact whatever the
// rejection rate.

#include <cstring>
#include <vector>

#include "abi_call.hpp"
#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

namespace fheg {

namespace {

constexpr int kMaxSeedLimbs = 64;

// FIPS 180-4 4.2.2: the first 32 bits of the fractional parts of the cube
// roots of the first 64 primes; 5.3.3: of the square roots of the first 8.
__constant__ uint32_t kShaK[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5, 0xd807aa98,
    0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174, 0xe49b69c1, 0xefbe4786,
    0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da, 0x983e5152, 0xa831c66d, 0xb00327c8,
    0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967, 0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13,
    0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85, 0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819,
    0xd6990624, 0xf40e3585, 0x106aa070, 0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a,
    0x5b9cca4f, 0x682e6ff3, 0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7,
    0xc67178f2};
__constant__ uint32_t kShaH0[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};

__device__ __forceinline__ uint32_t rotr32(uint32_t x, int r) { return __funnelshift_r(x, x, r); }
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return __funnelshift_l(x, x, r); }

// SHA-256 of one 32-byte message (a single padded block), returned as the
// ChaCha key: word i = bytes 4i .. 4i+3 of the digest, little-endian.
__device__ void seed_digest_key(const uint8_t* seed, uint32_t* key) {
  uint32_t w[64];
#pragma unroll
  for (int i = 0; i < 8; i++)
    w[i] = ((uint32_t)seed[4 * i] << 24) | ((uint32_t)seed[4 * i + 1] << 16) | ((uint32_t)seed[4 * i + 2] << 8) |
           (uint32_t)seed[4 * i + 3];
  w[8] = 0x80000000u;
#pragma unroll
  for (int i = 9; i < 15; i++) w[i] = 0;
  w[15] = 256;  // message length in bits
#pragma unroll
  for (int i = 16; i < 64; i++) {
    const uint32_t s0 = rotr32(w[i - 15], 7) ^ rotr32(w[i - 15], 18) ^ (w[i - 15] >> 3);
    const uint32_t s1 = rotr32(w[i - 2], 17) ^ rotr32(w[i - 2], 19) ^ (w[i - 2] >> 10);
    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
  }
  uint32_t a = kShaH0[0], b = kShaH0[1], c = kShaH0[2], d = kShaH0[3], e = kShaH0[4], f = kShaH0[5], g = kShaH0[6],
           h = kShaH0[7];
#pragma unroll
  for (int i = 0; i < 64; i++) {
    const uint32_t t1 = h + (rotr32(e, 6) ^ rotr32(e, 11) ^ rotr32(e, 25)) + ((e & f) ^ (~e & g)) + kShaK[i] + w[i];
    const uint32_t t2 = (rotr32(a, 2) ^ rotr32(a, 13) ^ rotr32(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
    h = g;
    g = f;
    f = e;
    e = d + t1;
    d = c;
    c = b;
    b = a;
    a = t1 + t2;
  }
  const uint32_t hv[8] = {a, b, c, d, e, f, g, h};
#pragma unroll
  for (int i = 0; i < 8; i++) key[i] = __byte_perm(kShaH0[i] + hv[i], 0, 0x0123);  // big-endian digest word
}

#define FHEG_CHACHA_QR(a, b, c, d) \
  x[a] += x[b];                    \
  x[d] = rotl32(x[d] ^ x[a], 16);  \
  x[c] += x[d];                    \
  x[b] = rotl32(x[b] ^ x[c], 12);  \
  x[a] += x[b];                    \
  x[d] = rotl32(x[d] ^ x[a], 8);   \
  x[c] += x[d];                    \
  x[b] = rotl32(x[b] ^ x[c], 7);

// Block `counter` of the ChaCha8 keystream of `key` (stream id 0).
__device__ __forceinline__ void chacha8_block(const uint32_t* key, uint64_t counter, uint32_t* out) {
  uint32_t x[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                    key[4],      key[5],      key[6],      key[7],      (uint32_t)counter, (uint32_t)(counter >> 32),
                    0u,          0u};
#pragma unroll
  for (int r = 0; r < 4; r++) {
    FHEG_CHACHA_QR(0, 4, 8, 12)
    FHEG_CHACHA_QR(1, 5, 9, 13)
    FHEG_CHACHA_QR(2, 6, 10, 14)
    FHEG_CHACHA_QR(3, 7, 11, 15)
    FHEG_CHACHA_QR(0, 5, 10, 15)
    FHEG_CHACHA_QR(1, 6, 11, 12)
    FHEG_CHACHA_QR(2, 7, 8, 13)
    FHEG_CHACHA_QR(3, 4, 9, 14)
  }
  const uint32_t k0[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                           key[4],      key[5],      key[6],      key[7],      (uint32_t)counter,
                           (uint32_t)(counter >> 32), 0u, 0u};
#pragma unroll
  for (int i = 0; i < 16; i++) out[i] = x[i] + k0[i];
}

struct SeedLimbs {
  uint64_t q[kMaxSeedLimbs];
  uint64_t thresh[kMaxSeedLimbs];  // (2^64 - q) mod q: draws whose low word is below it are rejected
  uint32_t limbs, logn;
};

__global__ void k_seed_keys(const uint8_t* seeds, uint32_t* keys, uint32_t* flags, uint64_t count) {
  const uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= count) return;
  seed_digest_key(seeds + 32 * b, keys + 8 * b);
  flags[b] = 0;
}

// One ChaCha block (8 draws) per thread, at the positions the draws take when
// none is rejected.
__global__ void k_seeded_fast(const __grid_constant__ SeedLimbs P, const uint32_t* keys, uint32_t* flags,
                              uint64_t* out, uint64_t stride, uint64_t blocks_per_poly, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint64_t b = gid / blocks_per_poly, blk = gid - b * blocks_per_poly;
  uint32_t key[8];
  const uint4 k0 = reinterpret_cast<const uint4*>(keys + 8 * b)[0];
  const uint4 k1 = reinterpret_cast<const uint4*>(keys + 8 * b)[1];
  key[0] = k0.x, key[1] = k0.y, key[2] = k0.z, key[3] = k0.w;
  key[4] = k1.x, key[5] = k1.y, key[6] = k1.z, key[7] = k1.w;
  uint32_t w[16];
  chacha8_block(key, blk, w);
  const uint64_t s0 = blk * 8;
  const uint32_t j = (uint32_t)(s0 >> P.logn);  // N >= 8: a block's draws share one limb
  const uint64_t q = P.q[j], th = P.thresh[j];
  uint64_t* o = out + b * stride + s0;
  bool rejected = false;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint64_t x = (uint64_t)w[2 * k] | ((uint64_t)w[2 * k + 1] << 32);
    rejected |= x * q < th;
    o[k] = __umul64hi(x, q);
  }
  if (rejected) flags[b] = 1;
}

// Exact walk for flagged polynomials: one warp per polynomial, draws in
// order, 32 per step; lane l evaluates draw d + l under the current limb's
// modulus and the accepted ones are written at their prefix-count positions.
// A draw is rejected with probability below 1/4 (thresh < q < 2^62), so a
// limb takes about N/24 steps at worst; the walk still stops after L*N steps
// (over 96% of 32 L N draws rejected) and marks the polynomial with flag 2.
__global__ void k_seeded_exact(const __grid_constant__ SeedLimbs P, const uint32_t* keys, uint32_t* flags,
                               uint64_t* out, uint64_t stride) {
  const uint64_t b = blockIdx.x;
  if (flags[b] == 0) return;
  const uint32_t lane = threadIdx.x;
  uint32_t key[8];
#pragma unroll
  for (int i = 0; i < 8; i++) key[i] = keys[8 * b + i];
  const uint32_t n = 1u << P.logn;
  uint64_t* o = out + b * stride;
  uint64_t d = 0;  // next draw
  uint64_t steps = 0;
  const uint64_t max_steps = (uint64_t)P.limbs << P.logn;
  for (uint32_t j = 0; j < P.limbs; j++) {
    const uint64_t q = P.q[j], th = P.thresh[j];
    uint32_t filled = 0;
    while (filled < n) {
      if (++steps > max_steps) {
        if (lane == 0) flags[b] = 2;
        return;
      }
      const uint64_t di = d + lane;
      uint32_t w[16];
      chacha8_block(key, di >> 3, w);
      const uint32_t k = (uint32_t)(di & 7);
      uint32_t lo = 0, hi = 0;
#pragma unroll
      for (int t = 0; t < 8; t++)
        if (t == (int)k) lo = w[2 * t], hi = w[2 * t + 1];
      const uint64_t x = (uint64_t)lo | ((uint64_t)hi << 32);
      const bool acc = x * q >= th;
      const uint32_t ballot = __ballot_sync(0xffffffffu, acc);
      const uint32_t rank = __popc(ballot & ((1u << lane) - 1));
      if (acc && filled + rank < n) o[((uint64_t)j << P.logn) + filled + rank] = __umul64hi(x, q);
      const uint32_t got = __popc(ballot);
      if (filled + got >= n) {
        const uint32_t need = n - filled;
        const uint32_t last = __ffs(__ballot_sync(0xffffffffu, acc && rank == need - 1)) - 1;
        d += last + 1;
        filled = n;
      } else {
        filled += got;
        d += 32;
      }
    }
  }
}

#undef FHEG_CHACHA_QR

unsigned grid_for(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

// Host ChaCha8 block (the same function as chacha8_block) for the c1 seeds of
// a seeded key.
uint32_t hrotl(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

void host_chacha8_block(const uint32_t* key, uint64_t counter, uint32_t* out) {
  const uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                           key[4],      key[5],      key[6],      key[7],      (uint32_t)counter,
                           (uint32_t)(counter >> 32), 0u, 0u};
  uint32_t x[16];
  std::memcpy(x, st, sizeof(x));
  auto qr = [&](int a, int b, int c, int d) {
    x[a] += x[b];
    x[d] = hrotl(x[d] ^ x[a], 16);
    x[c] += x[d];
    x[b] = hrotl(x[b] ^ x[c], 12);
    x[a] += x[b];
    x[d] = hrotl(x[d] ^ x[a], 8);
    x[c] += x[d];
    x[b] = hrotl(x[b] ^ x[c], 7);
  };
  for (int r = 0; r < 4; r++) {
    qr(0, 4, 8, 12);
    qr(1, 5, 9, 13);
    qr(2, 6, 10, 14);
    qr(3, 7, 11, 15);
    qr(0, 5, 10, 15);
    qr(1, 6, 11, 12);
    qr(2, 7, 8, 13);
    qr(3, 4, 9, 14);
  }
  for (int i = 0; i < 16; i++) out[i] = x[i] + st[i];
}

}  // namespace

void poly_random_from_seed(const Context& c, const uint8_t* seeds, uint64_t* out, uint64_t stride, uint64_t count,
                           Workspace& ws, cudaStream_t st) {
  if (c.L() > (size_t)kMaxSeedLimbs) throw Error(FHEG_ERR_UNSUPPORTED, "seeded polynomials support up to 64 moduli");
  if (c.N() < 8) throw Error(FHEG_ERR_UNSUPPORTED, "degree below 8");
  if (stride < c.L() * c.N()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "poly_stride below the polynomial size");
  if (count == 0) return;
  SeedLimbs P{};
  P.limbs = (uint32_t)c.L();
  P.logn = c.logn;
  for (size_t j = 0; j < c.L(); j++) {
    const uint64_t q = c.moduli[j];
    P.q[j] = q;
    P.thresh[j] = (0 - q) % q;
  }
  ws.reserve((count * 4 + count / 2 + 64) * 8);
  size_t off = 0;
  uint32_t* keys = reinterpret_cast<uint32_t*>(ws.take(count * 4, &off));
  uint32_t* flags = reinterpret_cast<uint32_t*>(ws.take(count / 2 + 1, &off));
  k_seed_keys<<<grid_for(count, 128), 128, 0, st>>>(seeds, keys, flags, count);
  after_launch("k_seed_keys");
  const uint64_t bpp = (c.L() * c.N()) / 8, total = bpp * count;
  k_seeded_fast<<<grid_for(total, 256), 256, 0, st>>>(P, keys, flags, out, stride, bpp, total);
  after_launch("k_seeded_fast");
  k_seeded_exact<<<(unsigned)count, 32, 0, st>>>(P, keys, flags, out, stride);
  after_launch("k_seeded_exact");
}

// fhe-util/src/lib.rs:22-55 `sample_vec_cbd` over the next_u64 stream of
// ChaCha8Rng::from_seed(seed) (the 32 seed bytes are the key, little-endian
// words; draw k joins keystream words 2k and 2k+1). The reference's bit pool
// takes each 64-bit draw above the bits it holds and cuts 4v bits per sample
// (v the variance): sample i is bits [4vi, 4vi + 4v) of the draws' little-endian
// bit stream, the popcount of its low 2v bits minus that of its high 2v. So
// 16 samples take exactly v draws: thread t makes samples 16t .. 16t + 15
// from draws vt .. vt + v - 1, which it computes (up to three ChaCha blocks)
// and stages in shared memory.
constexpr int kCbdThreads = 128;

__global__ void __launch_bounds__(kCbdThreads) k_sample_cbd(const uint8_t* seeds, uint32_t variance, uint32_t n,
                                                            uint64_t chunks_per_vec, uint64_t total, int64_t* out) {
  __shared__ uint64_t draws[kCbdThreads * 16];
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint64_t vec = gid / chunks_per_vec, chunk = gid - vec * chunks_per_vec;
  uint32_t key[8];
  const uint8_t* sd = seeds + 32 * vec;
#pragma unroll
  for (int i = 0; i < 8; i++)
    key[i] = (uint32_t)sd[4 * i] | ((uint32_t)sd[4 * i + 1] << 8) | ((uint32_t)sd[4 * i + 2] << 16) |
             ((uint32_t)sd[4 * i + 3] << 24);
  uint64_t* w = draws + threadIdx.x * 16;
  const uint64_t first = chunk * variance;  // first draw of the chunk
  uint32_t blk[16];
  uint64_t have = ~0ull;
  for (uint32_t k = 0; k < variance; k++) {
    const uint64_t d = first + k;
    if ((d >> 3) != have) {
      have = d >> 3;
      chacha8_block(key, have, blk);
    }
    const uint32_t o = 2 * (uint32_t)(d & 7);
    w[k] = (uint64_t)blk[o] | ((uint64_t)blk[o + 1] << 32);
  }
  const uint32_t nb = 4 * variance, half = 2 * variance;
  const uint64_t base = chunk * 16;
  const uint32_t m = n - base < 16 ? (uint32_t)(n - base) : 16u;
  for (uint32_t s = 0; s < m; s++) {
    const uint32_t off = s * nb, k = off >> 6, sh = off & 63;
    uint64_t v = w[k] >> sh;
    if (sh && sh + nb > 64) v |= w[k + 1] << (64 - sh);
    if (nb < 64) v &= (1ull << nb) - 1;
    out[vec * n + base + s] =
        (int64_t)__popcll(v & ((1ull << half) - 1)) - (int64_t)__popcll(v >> half);
  }
}

void sample_cbd_from_seed(const uint8_t* seeds, size_t variance, size_t n, size_t count, int64_t* out,
                          cudaStream_t st) {
  if (variance < 1 || variance > 16) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The variance should be between 1 and 16");
  if (n == 0 || count == 0) return;
  if (n > (1u << 30)) throw Error(FHEG_ERR_INVALID_ARGUMENT, "vector size above 2^30");
  const uint64_t chunks = (n + 15) / 16, total = chunks * count;
  k_sample_cbd<<<grid_for(total, kCbdThreads), kCbdThreads, 0, st>>>(seeds, (uint32_t)variance, (uint32_t)n, chunks,
                                                                     total, out);
  after_launch("k_sample_cbd");
}

std::vector<uint8_t> ksk_c1_seeds(const uint8_t* seed, size_t count) {
  // rand_chacha from_seed: key words little-endian; generate_c1 takes 32
  // bytes (8 words) per c1[i] with Rng::fill.
  uint32_t key[8];
  for (int i = 0; i < 8; i++)
    key[i] = (uint32_t)seed[4 * i] | ((uint32_t)seed[4 * i + 1] << 8) | ((uint32_t)seed[4 * i + 2] << 16) |
             ((uint32_t)seed[4 * i + 3] << 24);
  std::vector<uint8_t> out(32 * count);
  uint32_t blk[16];
  for (size_t w = 0; w < 8 * count; w++) {
    if (w % 16 == 0) host_chacha8_block(key, w / 16, blk);
    const uint32_t v = blk[w % 16];
    for (int k = 0; k < 4; k++) out[4 * w + k] = (uint8_t)(v >> (8 * k));
  }
  return out;
}

}  // namespace fheg

using namespace fheg;

FHEG_API int fheg_sample_cbd_from_seed(const uint8_t* d_seeds, size_t variance, size_t n, size_t count,
                                       int64_t* d_out, void* stream) {
  return abi_call([&] {
    abi_count(n);
    abi_count(count);
    abi_need((d_seeds && d_out) || !count || !n, "null input");
    sample_cbd_from_seed(d_seeds, variance, n, count, d_out, static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_poly_random_from_seed(const fheg_context* ctx, const uint8_t* d_seeds, uint64_t* d_out,
                                        size_t poly_stride, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && ((d_seeds && d_out) || !count), "null input");
    const Context& c = *ctx->c;
    poly_random_from_seed(c, d_seeds, d_out, poly_stride ? poly_stride : c.L() * c.N(), count, *ctx->ws,
                          static_cast<cudaStream_t>(stream));
  });
}
