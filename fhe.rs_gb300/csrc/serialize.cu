// Wire format of polynomials on the device: the coefficient payload of the
// reference's `Rq` message (fhe-math/src/rq/convert.rs:17-93). Every limb of
// the power-basis polynomial is bit-packed little-endian with the bit length
// of its modulus minus one (zq/mod.rs:783-793, fhe-util/src/lib.rs:57-135),
// and the limbs are concatenated. Ntt polynomials go through the power basis
// (inverse NTT before packing, forward NTT after unpacking), as the
// reference's conversion does.

#include <vector>

#include "fheg.h"
#include "handles.hpp"
#include "lib.hpp"

namespace fheg {

namespace {

constexpr int kMaxLimbs = 64;

struct PackLayout {
  uint32_t limbs, logn;
  uint64_t poly_bytes;  // payload of one polynomial
  uint64_t poly_chunks;  // 8-byte chunks of one payload, counted per limb (the last of a limb may be short)
  uint64_t offset[kMaxLimbs + 1];  // byte offset of limb j within a payload
  uint64_t chunk0[kMaxLimbs + 1];  // first chunk of limb j
  uint32_t nbits[kMaxLimbs];
  uint64_t q[kMaxLimbs];
};

PackLayout make_layout(const Context& c) {
  if (c.L() > (size_t)kMaxLimbs) throw Error(FHEG_ERR_UNSUPPORTED, "serialization supports up to 64 moduli");
  PackLayout lay{};
  lay.limbs = (uint32_t)c.L();
  lay.logn = c.logn;
  uint64_t off = 0, chunks = 0;
  for (size_t j = 0; j < c.L(); j++) {
    uint32_t nb = 0;
    while (nb < 64 && ((c.moduli[j] - 1) >> nb)) nb++;
    lay.nbits[j] = nb;
    lay.q[j] = c.moduli[j];
    lay.offset[j] = off;
    lay.chunk0[j] = chunks;
    const uint64_t bytes = ((uint64_t)c.N() * nb + 7) / 8;  // zq serialization_length
    off += bytes;
    chunks += (bytes + 7) / 8;
  }
  lay.offset[c.L()] = off;
  lay.chunk0[c.L()] = chunks;
  lay.poly_bytes = off;
  lay.poly_chunks = chunks;
  return lay;
}

// One 8-byte chunk of a limb's packed stream per thread: bits [64c, 64c + 64)
// gathered from the (at most 64 / nb + 2) coefficients they overlap, stored
// as one word when the destination is aligned, else byte by byte (a limb's
// last chunk may be short).
__global__ void k_pack(const __grid_constant__ PackLayout lay, const uint64_t* in, uint8_t* out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint64_t poly = gid / lay.poly_chunks;
  const uint64_t pos = gid - poly * lay.poly_chunks;
  uint32_t j = 0;
  while (j + 1 < lay.limbs && pos >= lay.chunk0[j + 1]) j++;
  const uint64_t c = pos - lay.chunk0[j];
  const uint64_t n = 1ull << lay.logn;
  const uint32_t nb = lay.nbits[j];
  const uint64_t mask = nb == 64 ? ~0ull : ((1ull << nb) - 1);
  const uint64_t* row = in + (poly * lay.limbs + j) * n;
  const uint64_t bit0 = c * 64;
  uint64_t word = 0;
  for (uint64_t k = bit0 / nb; k < n && k * nb < bit0 + 64; k++) {
    const uint64_t v = row[k] & mask;
    const int64_t sh = (int64_t)(k * nb) - (int64_t)bit0;  // position of v's bit 0 within the word
    if (sh >= 0) word |= v << sh;
    else word |= v >> (-sh);
  }
  const uint64_t limb_bytes = lay.offset[j + 1] - lay.offset[j];
  const uint64_t nbytes = limb_bytes - c * 8 < 8 ? limb_bytes - c * 8 : 8;
  uint8_t* dst = out + poly * lay.poly_bytes + lay.offset[j] + c * 8;
  if (nbytes == 8 && ((uintptr_t)dst & 7) == 0) {
    *reinterpret_cast<uint64_t*>(dst) = word;
  } else {
    for (uint64_t b = 0; b < nbytes; b++) dst[b] = (uint8_t)(word >> (8 * b));
  }
}

// One coefficient per thread: bits [k nb, k nb + nb) of the limb's stream
// (at most 9 bytes), reduced once modulo q_j.
__global__ void k_unpack(const __grid_constant__ PackLayout lay, const uint8_t* in, uint64_t* out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint64_t n = 1ull << lay.logn;
  const uint64_t k = gid & (n - 1);
  const uint64_t row = gid >> lay.logn;  // poly * limbs + j
  const uint32_t j = (uint32_t)(row % lay.limbs);
  const uint64_t poly = row / lay.limbs;
  const uint32_t nb = lay.nbits[j];
  const uint8_t* p = in + poly * lay.poly_bytes + lay.offset[j];
  const uint64_t limb_bytes = lay.offset[j + 1] - lay.offset[j];
  const uint64_t bit = k * nb;
  const uint64_t b0 = bit >> 3;
  const uint32_t s = (uint32_t)(bit & 7);
  uint64_t lo = 0, hi = 0;  // bytes b0 .. b0 + 8 as a 72-bit little-endian value
#pragma unroll
  for (int t = 0; t < 8; t++)
    if (b0 + t < limb_bytes) lo |= (uint64_t)p[b0 + t] << (8 * t);
  if (b0 + 8 < limb_bytes) hi = p[b0 + 8];
  uint64_t v = (lo >> s) | (s ? hi << (64 - s) : 0);
  if (nb < 64) v &= (1ull << nb) - 1;
  out[gid] = v >= lay.q[j] ? v - lay.q[j] : v;
}

unsigned nblk(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

}  // namespace

size_t poly_serialized_bytes(const Context& c) { return make_layout(c).poly_bytes; }

void poly_serialize(const Context& c, int representation, const uint64_t* polys, uint8_t* bytes, uint64_t count,
                    DevBuf& scratch, cudaStream_t st) {
  if (count == 0) return;
  const PackLayout lay = make_layout(c);
  const uint64_t* src = polys;
  if (representation == 1) {
    const size_t words = count * c.L() * c.N();
    scratch.reserve(words * 8);
    PolyRef in = plain_ref(const_cast<uint64_t*>(polys), c.L(), c.logn), tmp = plain_ref(scratch.u64(), c.L(), c.logn);
    ntt_backward(c, in, tmp, count, st);
    src = scratch.u64();
  }
  const uint64_t total = count * lay.poly_chunks;
  k_pack<<<nblk(total, 256), 256, 0, st>>>(lay, src, bytes, total);
  after_launch("k_pack");
}

void poly_deserialize(const Context& c, int representation, const uint8_t* bytes, uint64_t* polys, uint64_t count,
                      cudaStream_t st) {
  if (count == 0) return;
  const PackLayout lay = make_layout(c);
  const uint64_t total = count * c.L() << c.logn;
  k_unpack<<<nblk(total, 256), 256, 0, st>>>(lay, bytes, polys, total);
  after_launch("k_unpack");
  if (representation == 1) {
    PolyRef r = plain_ref(polys, c.L(), c.logn);
    ntt_forward(c, r, r, count, false, st);
  }
}

}  // namespace fheg

using namespace fheg;

namespace {

template <class F>
int guarded(F&& f) {
  try {
    set_last_error("");
    f();
    return FHEG_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return FHEG_ERR_INTERNAL;
  }
}

void need(bool cond, const char* what) {
  if (!cond) throw Error(FHEG_ERR_INVALID_ARGUMENT, what);
}

}  // namespace

FHEG_API int fheg_poly_serialized_size(const fheg_context* ctx, size_t* bytes) {
  return guarded([&] {
    need(ctx && bytes, "null input");
    *bytes = poly_serialized_bytes(*ctx->c);
  });
}

FHEG_API int fheg_poly_serialize(const fheg_context* ctx, int representation, const uint64_t* d_polys,
                                 uint8_t* d_bytes, size_t count, void* stream) {
  return guarded([&] {
    need(ctx && (representation == 0 || representation == 1), "bad context or representation");
    need((d_polys && d_bytes) || !count, "null input");
    DevBuf scratch;
    poly_serialize(*ctx->c, representation, d_polys, d_bytes, count, scratch, static_cast<cudaStream_t>(stream));
    if (scratch.ptr) check_cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
  });
}

FHEG_API int fheg_poly_deserialize(const fheg_context* ctx, int representation, const uint8_t* d_bytes,
                                   uint64_t* d_polys, size_t count, void* stream) {
  return guarded([&] {
    need(ctx && (representation == 0 || representation == 1), "bad context or representation");
    need((d_polys && d_bytes) || !count, "null input");
    poly_deserialize(*ctx->c, representation, d_bytes, d_polys, count, static_cast<cudaStream_t>(stream));
  });
}
