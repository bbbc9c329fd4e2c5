// Wire format of polynomials on the device: the coefficient payload of the
// reference's `Rq` message (fhe-math/src/rq/convert.rs:17-93). Every limb of
// the power-basis polynomial is bit-packed little-endian with the bit length
// of its modulus minus one (zq/mod.rs:783-793, fhe-util/src/lib.rs:57-135),
// and the limbs are concatenated. Ntt polynomials go through the power basis
// (inverse NTT before packing, forward NTT after unpacking), as the
// reference's conversion does.

#include <cstring>
#include <string>
#include <vector>

#include "fheg.h"
#include "handles.hpp"
#include "abi_call.hpp"
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
__global__ void k_pack(const __grid_constant__ PackLayout lay, const PolyRef in, uint8_t* out, uint64_t total) {
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
  const uint64_t* row = in.at((uint32_t)poly, j);
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
__global__ void k_unpack(const __grid_constant__ PackLayout lay, const uint8_t* in, const PolyRef out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint64_t n = 1ull << lay.logn;
  const uint64_t k = gid & (n - 1);
  const uint32_t row = row_of(gid, lay.logn);  // poly * limbs + j
  const uint32_t j = row % lay.limbs;
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
  out.at((uint32_t)poly, j)[k] = v >= lay.q[j] ? v - lay.q[j] : v;
}

unsigned nblk(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

}  // namespace

size_t poly_serialized_bytes(const Context& c) { return make_layout(c).poly_bytes; }

// Payloads of `count` polynomials read through `in` (Ntt polynomials go
// through `tmp`, count * L * N words, in the power basis) into `bytes`.
void pack_polys(const Context& c, int representation, PolyRef in, uint8_t* bytes, uint64_t count, uint64_t* tmp,
                cudaStream_t st) {
  if (count == 0) return;
  const PackLayout lay = make_layout(c);
  PolyRef src = in;
  if (representation >= 1) {  // Ntt and NttShoup values go through the power basis
    src = plain_ref(tmp, c.L(), c.logn);
    ntt_backward(c, in, src, count, st);
  }
  const uint64_t total = count * lay.poly_chunks;
  k_pack<<<nblk(total, 256), 256, 0, st>>>(lay, src, bytes, total);
  after_launch("k_pack");
}

// Payloads back into `count` polynomials written through `out`.
void unpack_polys(const Context& c, int representation, const uint8_t* bytes, PolyRef out, uint64_t count,
                  cudaStream_t st) {
  if (count == 0) return;
  const PackLayout lay = make_layout(c);
  const uint64_t total = count * c.L() << c.logn;
  k_unpack<<<nblk(total, 256), 256, 0, st>>>(lay, bytes, out, total);
  after_launch("k_unpack");
  if (representation >= 1) ntt_forward(c, out, out, count, false, st);
}

void poly_serialize(const Context& c, int representation, const uint64_t* polys, uint8_t* bytes, uint64_t count,
                    DevBuf& scratch, cudaStream_t st) {
  if (count == 0) return;
  if (representation >= 1) scratch.reserve(count * c.L() * c.N() * 8);
  pack_polys(c, representation, plain_ref(const_cast<uint64_t*>(polys), c.L(), c.logn), bytes, count,
             representation >= 1 ? scratch.u64() : nullptr, st);
}

void poly_deserialize(const Context& c, int representation, const uint8_t* bytes, uint64_t* polys, uint64_t count,
                      cudaStream_t st) {
  unpack_polys(c, representation, bytes, plain_ref(polys, c.L(), c.logn), count, st);
}

// ---------------------------------------------------------------------------
// Protobuf framing of `Rq` and `Ciphertext` messages (rq.proto, bfv.proto)
// as the reference writes them with prost: fields in tag order, proto3
// defaults (0, false, empty) left out, every element of a repeated field
// written; readers take fields in any order, the last value of a scalar
// wins, and unknown fields are skipped.

namespace {

constexpr uint64_t kReprCode[3] = {1, 2, 3};  // fheg representation -> rq.proto Representation

size_t varint_len(uint64_t v) {
  size_t n = 1;
  while (v >= 0x80) {
    v >>= 7;
    n++;
  }
  return n;
}

uint8_t* put_varint(uint8_t* p, uint64_t v) {
  while (v >= 0x80) {
    *p++ = (uint8_t)(v | 0x80);
    v >>= 7;
  }
  *p++ = (uint8_t)v;
  return p;
}

struct Span {
  const uint8_t* p = nullptr;
  size_t n = 0;
};

struct Field {
  uint32_t num, type;
  uint64_t value;  // varints
  Span bytes;      // length-delimited fields
};

// Iterates over the fields of one message.
struct Reader {
  const uint8_t* p;
  const uint8_t* end;
  const char* what;
  void fail(const char* why) const {
    throw Error(FHEG_ERR_INVALID_ARGUMENT, std::string(what) + " decode: " + why);
  }
  uint64_t varint() {
    uint64_t v = 0;
    for (int shift = 0; shift < 70; shift += 7) {
      if (p >= end) fail("truncated varint");
      const uint8_t c = *p++;
      if (shift == 63 && (c & 0x7e)) fail("varint overflow");
      v |= (uint64_t)(c & 0x7f) << shift;
      if (!(c & 0x80)) return v;
    }
    fail("varint too long");
    return 0;
  }
  bool next(Field& f) {
    if (p >= end) return false;
    const uint64_t key = varint();
    f.num = (uint32_t)(key >> 3);
    f.type = (uint32_t)(key & 7);
    if (f.num == 0) fail("field number 0");
    switch (f.type) {
      case 0: f.value = varint(); break;
      case 1:
        if (end - p < 8) fail("truncated fixed64");
        p += 8;
        break;
      case 2: {
        const uint64_t n = varint();
        if (n > (uint64_t)(end - p)) fail("truncated field");
        f.bytes = Span{p, (size_t)n};
        p += n;
        break;
      }
      case 5:
        if (end - p < 4) fail("truncated fixed32");
        p += 4;
        break;
      default: fail("unsupported wire type");
    }
    return true;
  }
  void expect(const Field& f, uint32_t type) const {
    if (f.type != type) fail("invalid wire type");
  }
};

// Length of one encoded Rq message of a polynomial over `c`.
size_t rq_message_len(const Context& c, bool avt) {
  const size_t payload = poly_serialized_bytes(c);
  return 2 + 1 + varint_len(c.N()) + 1 + varint_len(payload) + payload + (avt ? 2 : 0);
}

// Writes the Rq message of one packed payload; returns the end.
uint8_t* put_rq(uint8_t* o, const Context& c, int representation, const uint8_t* payload, bool avt) {
  const size_t n = poly_serialized_bytes(c);
  *o++ = 0x08;  // representation
  o = put_varint(o, kReprCode[representation]);
  *o++ = 0x10;  // degree
  o = put_varint(o, c.N());
  *o++ = 0x1a;  // coefficients
  o = put_varint(o, n);
  std::memcpy(o, payload, n);
  o += n;
  if (avt) {
    *o++ = 0x20;  // allow_variable_time
    *o++ = 1;
  }
  return o;
}

// The payload of one Rq message for a polynomial over `c` whose rq.proto
// representation must be `code` (convert.rs:44-135, parse_proto and
// TryConvertFrom<&Rq>).
Span parse_rq_code(Span m, const Context& c, uint64_t code) {
  Reader r{m.p, m.p + m.n, "Rq"};
  uint64_t repr = 0, degree = 0;
  Span coeffs;
  Field f;
  while (r.next(f)) {
    if (f.num == 1) r.expect(f, 0), repr = f.value;
    else if (f.num == 2) r.expect(f, 0), degree = f.value & 0xffffffffu;
    else if (f.num == 3) r.expect(f, 2), coeffs = f.bytes;
    else if (f.num == 4) r.expect(f, 0);
  }
  const int32_t rep = (int32_t)(uint32_t)repr;
  if (rep < 0 || rep > 3) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid representation");
  if (rep == 0) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Unknown representation");
  if ((uint64_t)rep != code)
    throw Error(FHEG_ERR_INVALID_ARGUMENT,
                "The representation asked for does not match the representation in the serialization");
  if (degree % 8 != 0 || degree < 8) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid degree");
  if (degree != c.N()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid degree: not the context's degree");
  if (coeffs.n != poly_serialized_bytes(c)) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid coefficients");
  return coeffs;
}

Span parse_rq(Span m, const Context& c, int representation) { return parse_rq_code(m, c, kReprCode[representation]); }

struct CtMessage {
  std::vector<Span> c;
  Span seed;
  uint64_t level = 0;
};

CtMessage parse_ct(const uint8_t* msg, size_t len) {
  Reader r{msg, msg + len, "Ciphertext"};
  CtMessage m;
  Field f;
  while (r.next(f)) {
    if (f.num == 1) r.expect(f, 2), m.c.push_back(f.bytes);
    else if (f.num == 2) r.expect(f, 2), m.seed = f.bytes;
    else if (f.num == 3) r.expect(f, 0), m.level = f.value & 0xffffffffu;
  }
  return m;
}

// ciphertext.rs:196-216: part count and level checks.
void check_ct(const Params& par, const CtMessage& m) {
  if (m.c.empty() || (m.c.size() == 1 && m.seed.n == 0))
    throw Error(FHEG_ERR_WRONG_PARTS, "Not enough polynomials");
  if (m.level > par.max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
  if (m.seed.n != 0 && m.seed.n != 32) throw Error(FHEG_ERR_INVALID_ARGUMENT, "InvalidSeedSize");
}

}  // namespace

size_t ciphertext_message_len(const Params& par, size_t level, size_t parts, bool seeded, bool avt) {
  const Context& c = *par.ctx(level);
  const size_t rq = rq_message_len(c, avt);
  const size_t stored = parts - (seeded ? 1 : 0);
  return stored * (1 + varint_len(rq) + rq) + (seeded ? 34 : 0) + (level ? 1 + varint_len(level) : 0);
}

void ciphertext_to_bytes(const Params& par, size_t level, size_t parts, const uint64_t* ct, uint64_t count,
                         const uint8_t* seeds, bool avt, uint8_t* out, Workspace& ws, cudaStream_t st) {
  if (parts < 1 || (seeds && parts < 2)) throw Error(FHEG_ERR_WRONG_PARTS, "Not enough polynomials");
  if (count == 0) return;
  const Context& c = *par.ctx(level);
  const size_t L = c.L(), N = c.N(), stored = parts - (seeds ? 1 : 0);
  const size_t payload = poly_serialized_bytes(c);
  const size_t polys = count * stored;
  ws.reserve((polys * L * N + (polys * payload + 7) / 8 + 64) * 8);
  size_t off = 0;
  uint64_t* tmp = ws.take(polys * L * N, &off);
  uint8_t* packed = reinterpret_cast<uint8_t*>(ws.take((polys * payload + 7) / 8, &off));
  pack_polys(c, 1, sub_ref(const_cast<uint64_t*>(ct), L, c.logn, (uint32_t)parts, 0, (uint32_t)stored), packed,
             polys, tmp, st);
  std::vector<uint8_t> h(polys * payload);
  check_cuda(cudaMemcpyAsync(h.data(), packed, h.size(), cudaMemcpyDeviceToHost, st), "D2H");
  check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  const size_t rq = rq_message_len(c, avt);
  uint8_t* o = out;
  for (uint64_t b = 0; b < count; b++) {
    for (size_t k = 0; k < stored; k++) {
      *o++ = 0x0a;  // c
      o = put_varint(o, rq);
      o = put_rq(o, c, 1, h.data() + (b * stored + k) * payload, avt);
    }
    if (seeds) {
      *o++ = 0x12;  // seed
      *o++ = 32;
      std::memcpy(o, seeds + 32 * b, 32);
      o += 32;
    }
    if (level) {
      *o++ = 0x18;  // level
      o = put_varint(o, level);
    }
  }
}

void ciphertext_peek(const Params& par, const uint8_t* msg, size_t len, size_t* level, size_t* parts, int* seeded) {
  const CtMessage m = parse_ct(msg, len);
  check_ct(par, m);
  *level = (size_t)m.level;
  *parts = m.c.size() + (m.seed.n ? 1 : 0);
  *seeded = m.seed.n ? 1 : 0;
}

void ciphertext_from_bytes(const Params& par, const uint8_t* const* msgs, const size_t* lens, uint64_t count,
                           size_t level, size_t parts, uint64_t* out, Workspace& ws, Workspace& seed_ws,
                           cudaStream_t st) {
  if (count == 0) return;
  const Context& c = *par.ctx(level);
  const size_t L = c.L(), N = c.N(), payload = poly_serialized_bytes(c);
  std::vector<CtMessage> m(count);
  for (uint64_t b = 0; b < count; b++) {
    if (!msgs[b]) throw Error(FHEG_ERR_INVALID_ARGUMENT, "null message");
    m[b] = parse_ct(msgs[b], lens[b]);
    check_ct(par, m[b]);
    if (m[b].level != level || m[b].c.size() + (m[b].seed.n ? 1 : 0) != parts)
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "message of another level or part count than the batch");
    if ((m[b].seed.n != 0) != (m[0].seed.n != 0))
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "a batch mixes seeded and unseeded ciphertexts");
  }
  const bool seeded = m[0].seed.n != 0;
  const size_t stored = parts - (seeded ? 1 : 0);
  std::vector<uint8_t> h(count * stored * payload + (seeded ? 32 * count : 0));
  for (uint64_t b = 0; b < count; b++) {
    for (size_t k = 0; k < stored; k++) {
      const Span pl = parse_rq(m[b].c[k], c, 1);
      std::memcpy(h.data() + (b * stored + k) * payload, pl.p, payload);
    }
    if (seeded) std::memcpy(h.data() + count * stored * payload + 32 * b, m[b].seed.p, 32);
  }
  ws.reserve((h.size() + 7) / 8 * 8 + 512);
  size_t off = 0;
  uint8_t* d = reinterpret_cast<uint8_t*>(ws.take((h.size() + 7) / 8, &off));
  check_cuda(cudaMemcpyAsync(d, h.data(), h.size(), cudaMemcpyHostToDevice, st), "H2D");
  unpack_polys(c, 1, d, sub_ref(out, L, c.logn, (uint32_t)parts, 0, (uint32_t)stored), count * stored, st);
  if (seeded)
    poly_random_from_seed(c, d + count * stored * payload, out + (parts - 1) * L * N, parts * L * N, count, seed_ws,
                          st);
  // The pageable source buffer must outlive the copy.
  check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
}

// KeySwitchingKey messages (bfv.proto; key_switching_key.rs:332-420): c0[i]
// (and c1[i] unless the key carries its seed) as NttShoup Rq messages over the
// key context, then the levels and the decomposition base. Wrapped in
// RelinearizationKey { ksk = 1 } or GaloisKey { ksk = 1, exponent = 2 }
// (relinearization_key.rs:109-127, galois_key.rs:127-149).
fheg_ksk* ksk_from_message(const fheg_params* par, const uint8_t* msg, size_t len, int kind, uint64_t* exponent) {
  const Params& p = *par->p;
  Span ksk{msg, len};
  uint64_t exp = 0;
  if (kind != 0) {
    Reader r{msg, msg + len, kind == 1 ? "RelinearizationKey" : "GaloisKey"};
    bool found = false;
    Field f;
    while (r.next(f)) {
      if (f.num == 1) r.expect(f, 2), ksk = f.bytes, found = true;
      else if (f.num == 2 && kind == 2) r.expect(f, 0), exp = f.value & 0xffffffffu;
    }
    if (!found) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid serialization");
  }
  std::vector<Span> c0, c1;
  Span seed;
  uint64_t ct_level = 0, ksk_level = 0, log_base = 0;
  {
    Reader r{ksk.p, ksk.p + ksk.n, "KeySwitchingKey"};
    Field f;
    while (r.next(f)) {
      if (f.num == 1) r.expect(f, 2), c0.push_back(f.bytes);
      else if (f.num == 2) r.expect(f, 2), c1.push_back(f.bytes);
      else if (f.num == 3) r.expect(f, 2), seed = f.bytes;
      else if (f.num == 4) r.expect(f, 0), ct_level = f.value & 0xffffffffu;
      else if (f.num == 5) r.expect(f, 0), ksk_level = f.value & 0xffffffffu;
      else if (f.num == 6) r.expect(f, 0), log_base = f.value & 0xffffffffu;
    }
  }
  if (ct_level > p.max_level() || ksk_level > p.max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
  // key_switching_key.rs:360-372: a decomposition base names the digit count
  // and needs both levels maximal.
  if (log_base != 0 && (ksk_level != p.max_level() || ct_level != p.max_level()))
    throw Error(FHEG_ERR_INVALID_ARGUMENT, "A decomposition size is specified but the levels are not maximal");
  if (log_base > 62) throw Error(FHEG_ERR_INVALID_ARGUMENT, "decomposition base above 2^62");
  const uint32_t log_modulus = log_modulus_of(p.moduli[0]);
  const size_t count = log_base ? (log_modulus + log_base - 1) / log_base : p.ctx(ct_level)->L();
  if (c0.size() != count) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Incorrect number of values in c0");
  if (seed.n == 0 && c1.size() != count) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Incorrect number of values in c1");
  if (seed.n != 0 && seed.n != 32) throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid seed");
  if (kind == 2) {
    const uint64_t two_n = 2 * p.ctx(ct_level)->N();
    if (exp % 2 == 0 || exp >= two_n)
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid exponent");  // SubstitutionExponent::new
  }
  fheg_ksk* h = new_ksk_handle(par, ct_level, ksk_level, nullptr, count, (int64_t)log_base);
  try {
    const Ksk& k = h->k;
    const Context& kc = *k.ctx_ksk;
    const size_t payload = poly_serialized_bytes(kc);
    const bool seeded = seed.n != 0;
    std::vector<uint8_t> hb((seeded ? 1 : 2) * count * payload);
    // NttShoup polynomials (representation 3): payloads in the power basis.
    for (size_t i = 0; i < count; i++) {
      std::memcpy(hb.data() + i * payload, parse_rq_code(c0[i], kc, 3).p, payload);
      if (!seeded) std::memcpy(hb.data() + (count + i) * payload, parse_rq_code(c1[i], kc, 3).p, payload);
    }
    DevBuf d(hb.size());
    upload(d.ptr, hb.data(), hb.size());
    const uint8_t* db = static_cast<const uint8_t*>(d.ptr);
    unpack_polys(kc, 1, db, plain_ref(k.values(0), kc.L(), kc.logn), count, nullptr);
    if (seeded) {
      h->k.seed.assign(seed.p, seed.p + 32);
      const std::vector<uint8_t> seeds = ksk_c1_seeds(seed.p, count);
      DevBuf ds(seeds.size());
      upload(ds.ptr, seeds.data(), seeds.size());
      Workspace ws;
      poly_random_from_seed(kc, static_cast<const uint8_t*>(ds.ptr), k.values(1), kc.L() * kc.N(), count, ws,
                            nullptr);
      check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    } else {
      unpack_polys(kc, 1, db + count * payload, plain_ref(k.values(1), kc.L(), kc.logn), count, nullptr);
    }
    check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
  } catch (...) {
    delete h;
    throw;
  }
  if (exponent) *exponent = exp;
  return h;
}

// Length-delimited field (wire type 2) header.
uint8_t* put_len_field(uint8_t* o, uint32_t field, size_t len) {
  o = put_varint(o, ((uint64_t)field << 3) | 2);
  return put_varint(o, len);
}
uint8_t* put_varint_field(uint8_t* o, uint32_t field, uint64_t v) {
  if (v == 0) return o;  // proto3 default left out
  o = put_varint(o, (uint64_t)field << 3);
  return put_varint(o, v);
}
size_t varint_field_len(uint32_t field, uint64_t v) {
  return v ? varint_len((uint64_t)field << 3) + varint_len(v) : 0;
}

// The KeySwitchingKey message of a device key (key_switching_key.rs:332-352):
// c0[i], then c1[i] or the seed, as NttShoup Rq messages whose payloads are
// the power basis of the key values (rq/convert.rs:17-42), with
// allow_variable_time set as on the reference's keys; then the levels and
// the decomposition base.
std::vector<uint8_t> ksk_message_bytes(const Ksk& k) {
  const Context& kc = *k.ctx_ksk;
  const size_t n = k.count, payload = poly_serialized_bytes(kc);
  const bool seeded = !k.seed.empty();
  const size_t polys = seeded ? n : 2 * n;  // c1 follows c0 in the key's buffer
  DevBuf tmp(polys * kc.L() * kc.N() * 8), packed(polys * payload);
  pack_polys(kc, 2, plain_ref(k.values(0), kc.L(), kc.logn), static_cast<uint8_t*>(packed.ptr), polys, tmp.u64(),
             nullptr);
  std::vector<uint8_t> hp(polys * payload);
  check_cuda(cudaMemcpy(hp.data(), packed.ptr, hp.size(), cudaMemcpyDeviceToHost), "D2H");
  const size_t rq = rq_message_len(kc, true);
  const size_t rq_field = 1 + varint_len(rq) + rq;
  const size_t len = polys * rq_field + (seeded ? 34 : 0) + varint_field_len(4, k.ciphertext_level) +
                     varint_field_len(5, k.ksk_level) + varint_field_len(6, k.log_base);
  std::vector<uint8_t> out(len);
  uint8_t* o = out.data();
  for (size_t i = 0; i < n; i++) {
    o = put_len_field(o, 1, rq);
    o = put_rq(o, kc, 2, hp.data() + i * payload, true);
  }
  if (seeded) {
    o = put_len_field(o, 3, 32);
    std::memcpy(o, k.seed.data(), 32);
    o += 32;
  } else {
    for (size_t i = 0; i < n; i++) {
      o = put_len_field(o, 2, rq);
      o = put_rq(o, kc, 2, hp.data() + (n + i) * payload, true);
    }
  }
  o = put_varint_field(o, 4, k.ciphertext_level);
  o = put_varint_field(o, 5, k.ksk_level);
  o = put_varint_field(o, 6, k.log_base);
  if ((size_t)(o - out.data()) != len) throw Error(FHEG_ERR_INTERNAL, "key message length");
  return out;
}

// RelinearizationKey { ksk = 1 } (relinearization_key.rs:109-115) or
// GaloisKey { ksk = 1, exponent = 2 } (galois_key.rs:127-134) around it.
std::vector<uint8_t> wrap_ksk(const std::vector<uint8_t>& ksk, int kind, uint64_t exponent) {
  if (kind == 0) return ksk;
  const size_t len = 1 + varint_len(ksk.size()) + ksk.size() + (kind == 2 ? varint_field_len(2, exponent) : 0);
  std::vector<uint8_t> out(len);
  uint8_t* o = put_len_field(out.data(), 1, ksk.size());
  std::memcpy(o, ksk.data(), ksk.size());
  o += ksk.size();
  if (kind == 2) o = put_varint_field(o, 2, exponent);
  return out;
}

void copy_out(const std::vector<uint8_t>& msg, uint8_t* h_out, size_t cap, size_t* len) {
  *len = msg.size();
  if (!h_out) return;
  if (cap < msg.size()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "output buffer too small for the message");
  std::memcpy(h_out, msg.data(), msg.size());
}

}  // namespace fheg

using namespace fheg;

FHEG_API int fheg_poly_serialized_size(const fheg_context* ctx, size_t* bytes) {
  return abi_call([&] {
    abi_need(ctx && bytes, "null input");
    *bytes = poly_serialized_bytes(*ctx->c);
  });
}

FHEG_API int fheg_poly_serialize(const fheg_context* ctx, int representation, const uint64_t* d_polys,
                                 uint8_t* d_bytes, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && representation >= 0 && representation <= 2, "bad context or representation");
    abi_need((d_polys && d_bytes) || !count, "null input");
    DevBuf scratch;
    poly_serialize(*ctx->c, representation, d_polys, d_bytes, count, scratch, static_cast<cudaStream_t>(stream));
    if (scratch.ptr) check_cuda(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), "cudaStreamSynchronize");
  });
}

FHEG_API int fheg_poly_deserialize(const fheg_context* ctx, int representation, const uint8_t* d_bytes,
                                   uint64_t* d_polys, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(ctx && representation >= 0 && representation <= 2, "bad context or representation");
    abi_need((d_polys && d_bytes) || !count, "null input");
    poly_deserialize(*ctx->c, representation, d_bytes, d_polys, count, static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_ciphertext_serialized_size(const fheg_params* par, size_t level, size_t parts, int seeded,
                                             int allow_variable_time, size_t* bytes) {
  return abi_call([&] {
    abi_need(par && bytes, "null input");
    if (level > par->p->max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    if (parts < 1 || (seeded && parts < 2)) throw Error(FHEG_ERR_WRONG_PARTS, "Not enough polynomials");
    *bytes = ciphertext_message_len(*par->p, level, parts, seeded != 0, allow_variable_time != 0);
  });
}

FHEG_API int fheg_ciphertext_to_bytes(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_ct,
                                      size_t count, const uint8_t* h_seeds, int allow_variable_time, uint8_t* h_out,
                                      size_t out_capacity, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((d_ct && h_out) || !count), "null input");
    if (level > par->p->max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    if (parts < 1 || (h_seeds && parts < 2)) throw Error(FHEG_ERR_WRONG_PARTS, "Not enough polynomials");
    const size_t one = ciphertext_message_len(*par->p, level, parts, h_seeds != nullptr, allow_variable_time != 0);
    abi_need(out_capacity >= count * one, "output buffer too small");
    ciphertext_to_bytes(*par->p, level, parts, d_ct, count, h_seeds, allow_variable_time != 0, h_out,
                        const_cast<fheg_params*>(par)->ws, static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_ciphertext_peek(const fheg_params* par, const uint8_t* h_msg, size_t len, size_t* level,
                                  size_t* parts, int* seeded) {
  return abi_call([&] {
    abi_need(par && h_msg && level && parts && seeded, "null input");
    ciphertext_peek(*par->p, h_msg, len, level, parts, seeded);
  });
}

FHEG_API int fheg_ciphertext_from_bytes(const fheg_params* par, const uint8_t* const* h_msgs, const size_t* lens,
                                        size_t count, size_t level, size_t parts, uint64_t* d_out, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((h_msgs && lens && d_out) || !count), "null input");
    if (level > par->p->max_level()) throw Error(FHEG_ERR_INVALID_LEVEL, "InvalidLevel");
    if (parts < 2) throw Error(FHEG_ERR_WRONG_PARTS, "Not enough polynomials");
    fheg_params* p = const_cast<fheg_params*>(par);
    ciphertext_from_bytes(*p->p, h_msgs, lens, count, level, parts, d_out, p->ws, *p->level_handles[level].ws,
                          static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_ksk_to_bytes(const fheg_ksk* key, int kind, size_t exponent, uint8_t* h_out, size_t cap,
                               size_t* len) {
  return abi_call([&] {
    abi_need(key && len && kind >= 0 && kind <= 2, "null input or bad kind");
    if (kind == 2 && (exponent % 2 == 0 || exponent >= 2 * key->k.ctx_ct->N()))
      throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid exponent");
    copy_out(wrap_ksk(ksk_message_bytes(key->k), kind, exponent), h_out, cap, len);
  });
}

FHEG_API int fheg_evaluation_key_to_bytes(const fheg_ksk* const* keys, const size_t* exponents, size_t count,
                                          size_t ciphertext_level, size_t evaluation_key_level, uint8_t* h_out,
                                          size_t cap, size_t* len) {
  return abi_call([&] {
    abi_count(count);
    abi_need(len && ((keys && exponents) || !count), "null input");
    // evaluation_key.rs:382-392: { repeated GaloisKey gk = 2; ciphertext_level = 3;
    // evaluation_key_level = 4 }, keys in the order given.
    std::vector<std::vector<uint8_t>> gks;
    size_t total = varint_field_len(3, ciphertext_level) + varint_field_len(4, evaluation_key_level);
    for (size_t i = 0; i < count; i++) {
      abi_need(keys[i] != nullptr, "null key");
      const Ksk& k = keys[i]->k;
      if (k.ciphertext_level != ciphertext_level || k.ksk_level != evaluation_key_level)
        throw Error(FHEG_ERR_KEY_MISMATCH, "Galois key at other levels than the evaluation key");
      if (exponents[i] % 2 == 0 || exponents[i] >= 2 * k.ctx_ct->N())
        throw Error(FHEG_ERR_INVALID_ARGUMENT, "Invalid exponent");
      gks.push_back(wrap_ksk(ksk_message_bytes(k), 2, exponents[i]));
      total += 1 + varint_len(gks.back().size()) + gks.back().size();
    }
    std::vector<uint8_t> out(total);
    uint8_t* o = out.data();
    for (const auto& g : gks) {
      o = put_len_field(o, 2, g.size());
      std::memcpy(o, g.data(), g.size());
      o += g.size();
    }
    o = put_varint_field(o, 3, ciphertext_level);
    o = put_varint_field(o, 4, evaluation_key_level);
    copy_out(out, h_out, cap, len);
  });
}

FHEG_API int fheg_evaluation_key_from_bytes(const fheg_params* par, const uint8_t* h_msg, size_t len,
                                            fheg_ksk** keys, size_t* exponents, size_t cap, size_t* count,
                                            size_t* ciphertext_level, size_t* evaluation_key_level) {
  return abi_call([&] {
    abi_need(par && h_msg && count, "null input");
    // evaluation_key.rs:394-432.
    std::vector<Span> gks;
    uint64_t ct_level = 0, ek_level = 0;
    {
      Reader r{h_msg, h_msg + len, "EvaluationKey"};
      Field f;
      while (r.next(f)) {
        if (f.num == 2) r.expect(f, 2), gks.push_back(f.bytes);
        else if (f.num == 3) r.expect(f, 0), ct_level = f.value & 0xffffffffu;
        else if (f.num == 4) r.expect(f, 0), ek_level = f.value & 0xffffffffu;
      }
    }
    *count = gks.size();
    if (ciphertext_level) *ciphertext_level = (size_t)ct_level;
    if (evaluation_key_level) *evaluation_key_level = (size_t)ek_level;
    if (!keys) return;
    abi_need(exponents != nullptr, "null exponents");
    if (cap < gks.size()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "too few key slots for the evaluation key");
    std::vector<fheg_ksk*> made;
    try {
      for (const Span& g : gks) {
        uint64_t e = 0;
        fheg_ksk* h = ksk_from_message(par, g.p, g.n, 2, &e);
        made.push_back(h);
        if (h->k.ciphertext_level != ct_level)
          throw Error(FHEG_ERR_INVALID_ARGUMENT, "Galois key has incorrect ciphertext level");
        if (h->k.ksk_level != ek_level)
          throw Error(FHEG_ERR_INVALID_ARGUMENT, "Galois key has incorrect evaluation key level");
        exponents[made.size() - 1] = (size_t)e;
      }
    } catch (...) {
      for (fheg_ksk* h : made) delete h;
      throw;
    }
    for (size_t i = 0; i < made.size(); i++) keys[i] = made[i];
  });
}

FHEG_API int fheg_ksk_from_bytes(const fheg_params* par, const uint8_t* h_msg, size_t len, int kind,
                                 fheg_ksk** out, size_t* exponent, size_t* ciphertext_level, size_t* ksk_level) {
  return abi_call([&] {
    abi_need(par && h_msg && out && kind >= 0 && kind <= 2, "null input or bad kind");
    uint64_t e = 0;
    fheg_ksk* h = ksk_from_message(par, h_msg, len, kind, &e);
    if (exponent) *exponent = (size_t)e;
    if (ciphertext_level) *ciphertext_level = h->k.ciphertext_level;
    if (ksk_level) *ksk_level = h->k.ksk_level;
    *out = h;
  });
}
