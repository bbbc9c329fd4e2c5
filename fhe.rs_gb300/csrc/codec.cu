// Plaintext side of the BFV path on the device: SIMD / coefficient encoding
// into the Ntt polynomial a Plaintext carries, ciphertext x plaintext
// products, and decryption with decoding.
//
//   encode   (plaintext_vec.rs:40-100): values -> [SIMD: scatter by
//            matrix_reps_index_map, inverse NTT mod t] -> lift into the
//            ciphertext context -> forward NTT          (Plaintext::poly_ntt)
//   mul      (ops/mod.rs:229-258): every part times poly_ntt
//   decrypt  (secret_key.rs:200-252): phase c0 + c1 s + c2 s^2 ... (Ntt) ->
//            inverse NTT -> t/Q scaling into the plaintext context ->
//            ((d + t) mod q_0) mod t -> [SIMD: forward NTT mod t, gather]

#include <mutex>

#include "fheg.h"
#include "handles.hpp"
#include "abi_call.hpp"
#include "lib.hpp"
#include "ntt.cuh"

namespace fheg {

namespace {

// parameters.rs:616-629: the SIMD slot map (SEAL's batch encoder order).
std::vector<uint32_t> index_map(size_t n) {
  uint32_t logn = 0;
  while (((size_t)1 << logn) < n) logn++;
  const size_t row = n >> 1, m = n << 1;
  size_t pos = 1;
  std::vector<uint32_t> map(n);
  auto brev = [&](size_t x) {
    size_t r = 0;
    for (uint32_t b = 0; b < logn; b++) r |= ((x >> b) & 1) << (logn - 1 - b);
    return (uint32_t)r;
  };
  for (size_t i = 0; i < row; i++) {
    map[i] = brev((pos - 1) >> 1);
    map[row | i] = brev((m - pos - 1) >> 1);
    pos = (pos * 3) & (m - 1);
  }
  return map;
}

// Values (< t) of polynomial `poly`, optionally gathered through a map:
// element i is values[map[i]] (the SIMD scatter v[map[k]] = values[k] read
// through the inverse map).
struct SrcValues {
  const uint64_t* values;  // [count][N]
  const uint32_t* map;     // null: identity
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return values[((uint64_t)j.poly << logn) + (map ? map[i] : i)];
  }
};

// Power-basis values v < t (one row per polynomial) lifted into every limb
// of the ciphertext context: v mod q_j, lazily reduced ([0, 2 q_j)).
struct SrcLift {
  const uint64_t* v;  // [count][N]
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    return reduce64_lazy(v[((uint64_t)j.poly << logn) + i], pr);
  }
};

// Phase c_0 + c_1 s + c_2 s^2 + ... of ciphertext j.poly at limb j.limb
// (Ntt), s the secret key's Ntt form (level-0 limbs; a level's context is a
// prefix of the top one).
struct SrcPhase {
  PolyRef ct;  // poly b * parts + k
  const uint64_t* s;
  uint32_t parts, logn;
  __device__ __forceinline__ void prefetch(const NttJob& j, uint32_t i) const {
    for (uint32_t k = 0; k < parts; k++) prefetch_l2(ct.at(j.poly * parts + k, j.limb) + i);
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint64_t sj = s[((uint64_t)j.limb << logn) + i];
    uint64_t acc = ct.at(j.poly * parts, j.limb)[i];
    uint64_t si = sj;
    for (uint32_t k = 1; k < parts; k++) {
      acc = add_mod(acc, mul_mod(ct.at(j.poly * parts + k, j.limb)[i], si, pr), pr.p);
      if (k + 1 < parts) si = mul_mod(si, sj, pr);
    }
    return acc;
  }
};

// secret_key.rs:233-245: ((d + t) mod q_0) mod t of the scaled phase's
// first limb.
struct SrcFinish {
  const uint64_t* d;  // [count][N]
  uint64_t t, q0;
  uint32_t logn;
  __device__ __forceinline__ uint64_t value(uint32_t poly, uint32_t i) const {
    return ((d[((uint64_t)poly << logn) + i] + t) % q0) % t;
  }
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime&, uint32_t i) const {
    return value(j.poly, i);
  }
};

// plaintext.rs:379-386: slot i of the decoded vector is NTT output
// map[i], so output j goes to slot inv[j].
struct DstSlots {
  uint64_t* out;       // [count][N]
  const uint32_t* inv;
  uint32_t logn;
  __device__ __forceinline__ void operator()(const NttJob& j, const DevPrime&, uint32_t i, uint64_t v) const {
    out[((uint64_t)j.poly << logn) + inv[i]] = v;
  }
  // Two-pass transforms store their intermediate through the same map.
  __device__ __forceinline__ uint64_t reload(const NttJob& j, uint32_t i) const {
    return out[((uint64_t)j.poly << logn) + inv[i]];
  }
};

// Encryption source (secret_key.rs:102-123 with plaintext.rs:71-98): the
// power-basis element e_i + Delta_j * ((v_i * (Q mod t)) mod t) of limb j,
// whose forward NTT is e_ntt + m_poly by linearity (Delta is a constant
// polynomial: Delta_j = (-t)^-1 mod q_j, parameters.rs:509-559).
struct SrcEncrypt {
  const int64_t* e;   // [count][N]
  const uint64_t* v;  // [count][N], < t
  const ulonglong2* delta;  // (Delta_j, Shoup) per limb
  uint64_t t, q_mod_t;
  uint32_t logn;
  __device__ __forceinline__ uint64_t operator()(const NttJob& j, const DevPrime& pr, uint32_t i) const {
    const uint64_t k = ((uint64_t)j.poly << logn) + i;
    const uint64_t m = (uint64_t)(((unsigned __int128)v[k] * q_mod_t) % t);
    const int64_t ei = e[k];
    const uint64_t ev = ei >= 0 ? (uint64_t)ei % pr.p : (pr.p - (uint64_t)(-(ei + 1)) % pr.p - 1);
    const ulonglong2 d = delta[j.limb];
    return add_mod(ev, mul_shoup(m % pr.p, d.x, d.y, pr.p), pr.p);
  }
};

// b -= a s and the copy of a: ciphertext (b, a), one thread per residue.
__global__ void k_encrypt_finish(const DevPrime* primes, uint64_t* out, const uint64_t* a, const uint64_t* s,
                                 uint32_t limbs, uint32_t logn, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t row = row_of(gid, logn);  // poly * limbs + limb
  const uint32_t limb = row % limbs;
  const uint64_t poly = row / limbs;
  const DevPrime pr = primes[limb];
  const uint64_t ai = a[gid];
  const uint64_t as = mul_mod(ai, s[((uint64_t)limb << logn) + i], pr);
  uint64_t* o = out + ((poly * 2 * limbs + limb) << logn) + i;
  o[0] = sub_mod(o[0], as, pr.p);
  o[(uint64_t)limbs << logn] = ai;
}

__global__ void k_finish(SrcFinish f, uint64_t* out, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  out[gid] = f.value((uint32_t)(gid >> f.logn), (uint32_t)(gid & ((1u << f.logn) - 1)));
}

__global__ void k_mul_plain(const DevPrime* primes, PolyRef ct, PolyRef pt, PolyRef out, uint32_t parts,
                            uint32_t limbs, uint32_t logn, uint32_t pt_per_ct, uint64_t total) {
  const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const uint32_t i = gid & ((1u << logn) - 1);
  const uint32_t job = row_of(gid, logn);
  const uint32_t limb = job % limbs;
  const uint32_t poly = job / limbs;  // b * parts + k
  const uint32_t b = poly / parts;
  const DevPrime pr = primes[limb];
  out.at(poly, limb)[i] = mul_mod(ct.at(poly, limb)[i], pt.at(pt_per_ct ? b : 0, limb)[i], pr);
}

unsigned nblk(uint64_t total, unsigned threads) { return (unsigned)((total + threads - 1) / threads); }

}  // namespace

const PlainSide& Params::plain_side() const {
  std::lock_guard<std::mutex> lock(plain_mu);
  if (plain) return *plain;
  auto ps = std::make_unique<PlainSide>();
  const size_t n = degree;
  if (supports_ntt(plaintext, n)) {
    ps->tctx = std::make_shared<Context>(std::vector<uint64_t>{plaintext}, n, nullptr);
    const std::vector<uint32_t> map = index_map(n);
    std::vector<uint32_t> both(2 * n);
    for (size_t i = 0; i < n; i++) {
      both[i] = map[i];
      both[n + map[i]] = (uint32_t)i;
    }
    ps->maps.alloc(both.size() * 4);
    upload(ps->maps.ptr, both.data(), both.size() * 4);
  }
  // parameters.rs:480-494: enough leading moduli for t plus 60 bits.
  size_t t_bits = 0;
  while (t_bits < 64 && (plaintext >> t_bits)) t_bits++;
  size_t acc = 0, count = 0;
  for (uint64_t q : moduli) {
    size_t bits = 0;
    while (bits < 64 && (q >> bits)) bits++;
    acc += bits;
    count++;
    if (acc >= t_bits + 60) break;
  }
  count = std::max<size_t>(1, std::min(count, moduli.size()));
  ps->plain_ctx = levels[0]->prefix(count);
  // parameters.rs:509-559: per level, the scaler cipher ctx -> plaintext ctx by t / Q_level.
  for (size_t l = 0; l < levels.size(); l++)
    ps->dec.push_back(std::make_unique<Scaler>(levels[l], ps->plain_ctx, BigUint(plaintext), levels[l]->rns->product));
  plain = std::move(ps);
  return *plain;
}

void plaintext_encode(const Params& par, size_t level, const uint64_t* values, bool simd, uint64_t* pt_ntt,
                      uint64_t count, Workspace& ws, cudaStream_t st) {
  if (count == 0) return;
  const PlainSide& ps = par.plain_side();
  const Context& c = *par.ctx(level);
  const uint32_t logn = c.logn;
  const uint64_t* v = values;
  if (simd) {
    if (!ps.tctx) throw Error(FHEG_ERR_UNSUPPORTED, "the plaintext modulus does not support SIMD encoding");
    ws.reserve(count * c.N() * 8 + 256);
    size_t off = 0;
    uint64_t* tmp = ws.take(count * c.N(), &off);
    const uint32_t* inv = static_cast<const uint32_t*>(ps.maps.ptr) + c.N();
    NttGeom gt{ps.tctx->primes_dev(), 1, 0};
    ntt_inverse_any(logn, gt, count, SrcValues{values, inv, logn}, DstPoly{plain_ref(tmp, 1, logn)}, st);
    v = tmp;
  }
  NttGeom g{c.primes_dev(), (uint32_t)c.L(), 0};
  ntt_forward_any<true>(logn, g, count, SrcLift{v, logn}, DstPoly{plain_ref(pt_ntt, c.L(), logn)}, st);
}

void ciphertext_mul_plain(const Params& par, size_t level, size_t parts, const uint64_t* ct, const uint64_t* pt,
                          bool pt_per_ct, uint64_t* out, uint64_t count, cudaStream_t st) {
  const Context& c = *par.ctx(level);
  const uint64_t total = count * parts * c.L() << c.logn;
  if (total == 0) return;
  k_mul_plain<<<nblk(total, 256), 256, 0, st>>>(c.primes_dev(), plain_ref(const_cast<uint64_t*>(ct), c.L(), c.logn),
                                                plain_ref(const_cast<uint64_t*>(pt), c.L(), c.logn),
                                                plain_ref(out, c.L(), c.logn), (uint32_t)parts, (uint32_t)c.L(),
                                                c.logn, pt_per_ct ? 1u : 0u, total);
  after_launch("k_mul_plain");
}

void encrypt(const SecretKeyDev& sk, size_t level, const uint64_t* values, bool simd, const uint64_t* a,
             const int64_t* e, uint64_t* out, uint64_t count, Workspace& ws, cudaStream_t st) {
  if (count == 0) return;
  const Params& par = *sk.par;
  const PlainSide& ps = par.plain_side();
  const Context& c = *par.ctx(level);
  const uint32_t logn = c.logn;
  const uint64_t t = par.plaintext;
  const size_t L = c.L();
  // Delta_j = (-t)^-1 mod q_j and Q mod t of this level (parameters.rs:509-559).
  std::vector<uint64_t> dh(2 * L);
  for (size_t j = 0; j < L; j++) {
    const uint64_t q = c.moduli[j];
    const uint64_t neg_t = (q - t % q) % q;
    dh[2 * j] = invmod(neg_t, q);
    dh[2 * j + 1] = shoup(dh[2 * j], q);
  }
  const uint64_t q_mod_t = c.rns->product.mod_u64(t);
  ws.reserve((count * c.N() + 2 * L) * 8 + 512);
  size_t off = 0;
  uint64_t* vbuf = ws.take(count * c.N(), &off);
  uint64_t* dbuf = ws.take(2 * L, &off);
  check_cuda(cudaMemcpyAsync(dbuf, dh.data(), dh.size() * 8, cudaMemcpyHostToDevice, st), "H2D");
  const uint64_t* v = values;
  if (simd) {
    if (!ps.tctx) throw Error(FHEG_ERR_UNSUPPORTED, "the plaintext modulus does not support SIMD encoding");
    const uint32_t* inv = static_cast<const uint32_t*>(ps.maps.ptr) + c.N();
    NttGeom gt{ps.tctx->primes_dev(), 1, 0};
    ntt_inverse_any(logn, gt, count, SrcValues{values, inv, logn}, DstPoly{plain_ref(vbuf, 1, logn)}, st);
    v = vbuf;
  }
  NttGeom g{c.primes_dev(), (uint32_t)L, 0};
  ntt_forward_any<true>(logn, g, count,
                        SrcEncrypt{e, v, reinterpret_cast<const ulonglong2*>(dbuf), t, q_mod_t, logn},
                        DstPoly{sub_ref(out, L, logn, 2, 0, 1)}, st);
  const uint64_t total = count * L << logn;
  k_encrypt_finish<<<nblk(total, 256), 256, 0, st>>>(c.primes_dev(), out, a, sk.s_ntt.u64(), (uint32_t)L, logn,
                                                     total);
  after_launch("k_encrypt_finish");
}

size_t decrypt_scratch_bytes(const Params& par, size_t level, uint64_t count) {
  const Context& c = *par.ctx(level);
  return (count * c.L() * c.N() + count * c.N()) * 8 + 2 * 256;
}

void decrypt(const SecretKeyDev& sk, size_t level, size_t parts, const uint64_t* ct, bool simd, uint64_t* values,
             uint64_t count, Workspace& ws, cudaStream_t st) {
  if (count == 0) return;
  const Params& par = *sk.par;
  const PlainSide& ps = par.plain_side();
  const Context& c = *par.ctx(level);
  const uint32_t logn = c.logn;
  if (parts < 2) throw Error(FHEG_ERR_WRONG_PARTS, "a ciphertext has at least two parts");
  if (simd && !ps.tctx) throw Error(FHEG_ERR_UNSUPPORTED, "the plaintext modulus does not support SIMD encoding");
  ws.reserve(decrypt_scratch_bytes(par, level, count));
  size_t off = 0;
  uint64_t* pb = ws.take(count * c.L() * c.N(), &off);
  uint64_t* d0 = ws.take(count * c.N(), &off);
  // Phase into the power basis.
  NttGeom g{c.primes_dev(), (uint32_t)c.L(), 0};
  ntt_inverse_any(logn, g, count,
                  SrcPhase{plain_ref(const_cast<uint64_t*>(ct), c.L(), logn), sk.s_ntt.u64(), (uint32_t)parts, logn},
                  DstPoly{plain_ref(pb, c.L(), logn)}, st);
  // t/Q scaling; only the first plaintext-context limb is read afterwards.
  const Scaler& sc = *ps.dec[level];
  rns_scale(*sc.rns, logn, plain_ref(pb, c.L(), logn), plain_ref(d0, 1, logn), 0, 1, count, st);
  const SrcFinish fin{d0, par.plaintext, par.moduli[0], logn};
  if (!simd) {
    const uint64_t total = count << logn;
    k_finish<<<nblk(total, 256), 256, 0, st>>>(fin, values, total);
    after_launch("k_finish");
    return;
  }
  const uint32_t* inv = static_cast<const uint32_t*>(ps.maps.ptr) + c.N();
  NttGeom gt{ps.tctx->primes_dev(), 1, 0};
  ntt_forward_any<true>(logn, gt, count, fin, DstSlots{values, inv, logn}, st);
}

}  // namespace fheg

using namespace fheg;

FHEG_API int fheg_plaintext_encode(const fheg_params* par, size_t level, const uint64_t* d_values, int simd,
                                   uint64_t* d_pt_ntt, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && ((d_values && d_pt_ntt) || !count), "null input");
    plaintext_encode(*par->p, level, d_values, simd != 0, d_pt_ntt, count, const_cast<fheg_params*>(par)->ws,
                     static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_ciphertext_mul_plain(const fheg_params* par, size_t level, size_t parts, const uint64_t* d_ct,
                                       const uint64_t* d_pt_ntt, int pt_per_ciphertext, uint64_t* d_out,
                                       size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(par && parts >= 1 && ((d_ct && d_pt_ntt && d_out) || !count), "null input");
    ciphertext_mul_plain(*par->p, level, parts, d_ct, d_pt_ntt, pt_per_ciphertext != 0, d_out, count,
                         static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_secret_key_create(const fheg_params* par, const int64_t* coeffs, fheg_secret_key** out) {
  return abi_call([&] {
    abi_need(par && coeffs && out, "null input");
    const Params& p = *par->p;
    const Context& c = *p.ctx(0);
    const size_t L = c.L(), N = c.N();
    // Poly::try_convert_from(&[i64], ctx) (rq/convert.rs): signed values into residues.
    std::vector<uint64_t> h(L * N);
    for (size_t j = 0; j < L; j++) {
      const uint64_t q = c.moduli[j];
      for (size_t i = 0; i < N; i++) {
        const int64_t v = coeffs[i];
        const uint64_t a = v < 0 ? (uint64_t)(-(v + 1)) + 1 : (uint64_t)v;
        const uint64_t r = a % q;
        h[j * N + i] = v < 0 ? (r ? q - r : 0) : r;
      }
    }
    auto sk = std::make_unique<fheg_secret_key>();
    sk->k.par = &p;
    sk->k.s_ntt.alloc(L * N * 8);
    upload(sk->k.s_ntt.ptr, h.data(), L * N * 8);
    PolyRef r = plain_ref(sk->k.s_ntt.u64(), L, c.logn);
    ntt_forward(c, r, r, 1, false, nullptr);
    check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
    *out = sk.release();
  });
}

FHEG_API void fheg_secret_key_destroy(fheg_secret_key* sk) { delete sk; }

FHEG_API int fheg_encrypt(const fheg_secret_key* sk, size_t level, const uint64_t* d_values, int simd,
                          const uint64_t* d_a, const int64_t* d_e, uint64_t* d_ct, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(sk && ((d_values && d_a && d_e && d_ct) || !count), "null input");
    encrypt(sk->k, level, d_values, simd != 0, d_a, d_e, d_ct, count, sk->ws, static_cast<cudaStream_t>(stream));
  });
}

FHEG_API int fheg_decrypt(const fheg_secret_key* sk, size_t level, size_t parts, const uint64_t* d_ct, int simd,
                          uint64_t* d_values, size_t count, void* stream) {
  return abi_call([&] {
    abi_count(count);
    abi_need(sk && ((d_ct && d_values) || !count), "null input");
    decrypt(sk->k, level, parts, d_ct, simd != 0, d_values, count, sk->ws, static_cast<cudaStream_t>(stream));
  });
}
