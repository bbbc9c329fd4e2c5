// CPU oracle for the fhe.rs RNS-BFV ciphertext hot path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, loop by loop, the CPU code of
// the reference crates `fhe-math` and `fhe` so that the GPU library can be
// checked bit for bit against it. Only tests, the smoke check and the CPU
// baseline leg of the benchmark load it; the GPU product never links it.
//
// Every function names the reference file:line it follows. Paths are relative
// to the reference repository root.
//
// Constants that need arbitrary precision (Barrett constants, RNS scaler
// theta values, NTT roots) are computed by the Python half of the oracle
// (oracle/ora.py) and passed in.

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

typedef unsigned __int128 u128;

namespace {

// fhe-math/src/zq/mod.rs:31-40 (`Modulus`): the fields the loops use.
struct Modulus {
  uint64_t p;
  uint64_t barrett_hi;
  uint64_t barrett_lo;
  uint64_t leading_zeros;
  uint64_t supports_opt;
};

// zq/mod.rs:659-668 `reduce1`: x in [0, 2p) -> x mod p.
inline uint64_t reduce1(uint64_t x, uint64_t p) { return x >= p ? x - p : x; }

// zq/mod.rs:693-707 `lazy_reduce_u128`: Barrett reduction into [0, 2p).
inline uint64_t lazy_reduce_u128(const Modulus& m, u128 a) {
  uint64_t a_lo = (uint64_t)a;
  uint64_t a_hi = (uint64_t)(a >> 64);
  u128 p_lo_lo = ((u128)a_lo * m.barrett_lo) >> 64;
  u128 p_hi_lo = (u128)a_hi * m.barrett_lo;
  u128 p_lo_hi = (u128)a_lo * m.barrett_hi;
  u128 q = ((p_lo_hi + p_hi_lo + p_lo_lo) >> 64) + (u128)a_hi * m.barrett_hi;
  return (uint64_t)(a - q * (u128)m.p);
}

// zq/mod.rs:594-596 `reduce_u128`.
inline uint64_t reduce_u128(const Modulus& m, u128 a) { return reduce1(lazy_reduce_u128(m, a), m.p); }

// zq/mod.rs:712-723 `lazy_reduce`.
inline uint64_t lazy_reduce(const Modulus& m, uint64_t a) {
  u128 p_lo_lo = ((u128)a * m.barrett_lo) >> 64;
  u128 p_lo_hi = (u128)a * m.barrett_hi;
  u128 q = (p_lo_hi + p_lo_lo) >> 64;
  return (uint64_t)((u128)a - q * (u128)m.p);
}

// zq/mod.rs:623-626 `reduce`.
inline uint64_t reduce(const Modulus& m, uint64_t a) { return reduce1(lazy_reduce(m, a), m.p); }

// zq/mod.rs:730-740 `lazy_reduce_opt_u128`.
inline uint64_t lazy_reduce_opt_u128(const Modulus& m, u128 a) {
  u128 q = (((u128)m.barrett_lo * (a >> 64)) + (a << m.leading_zeros)) >> 64;
  return (uint64_t)(a - q * (u128)m.p);
}

// zq/mod.rs:744-752 `lazy_reduce_opt`.
inline uint64_t lazy_reduce_opt(const Modulus& m, uint64_t a) {
  uint64_t q = a >> (64 - m.leading_zeros);
  return (uint64_t)((u128)a - (u128)q * (u128)m.p);
}

// zq/mod.rs:131-156 `mul` / `mul_opt` as selected by `mul_vec` (332-344).
inline uint64_t mul(const Modulus& m, uint64_t a, uint64_t b) {
  u128 x = (u128)a * b;
  if (m.supports_opt) return reduce1(lazy_reduce_opt_u128(m, x), m.p);
  return reduce_u128(m, x);
}

// zq/mod.rs:195-199 `shoup`.
inline uint64_t shoup(const Modulus& m, uint64_t a) { return (uint64_t)(((u128)a << 64) / m.p); }

// zq/mod.rs:224-234 `lazy_mul_shoup`: result in [0, 2p).
inline uint64_t lazy_mul_shoup(const Modulus& m, uint64_t a, uint64_t b, uint64_t b_shoup) {
  u128 q = ((u128)a * b_shoup) >> 64;
  return (uint64_t)((u128)a * b - q * (u128)m.p);
}

// zq/mod.rs:205-207 `mul_shoup`.
inline uint64_t mul_shoup(const Modulus& m, uint64_t a, uint64_t b, uint64_t b_shoup) {
  return reduce1(lazy_mul_shoup(m, a, b, b_shoup), m.p);
}

// ntt/native.rs:15-26 `NttOperator`.
struct NttOp {
  Modulus m;
  size_t n;
  const uint64_t* omegas;
  const uint64_t* omegas_shoup;
  const uint64_t* zetas_inv;
  const uint64_t* zetas_inv_shoup;
  uint64_t size_inv;
  uint64_t size_inv_shoup;
};

// native.rs:256-269 `butterfly`.
inline void butterfly(const NttOp& op, uint64_t& x, uint64_t& y, uint64_t w, uint64_t w_shoup) {
  uint64_t p2 = op.m.p * 2;
  x = reduce1(x, p2);
  uint64_t t = lazy_mul_shoup(op.m, y, w, w_shoup);
  y = x + p2 - t;
  x += t;
}

// native.rs:288-300 `inv_butterfly`.
inline void inv_butterfly(const NttOp& op, uint64_t& x, uint64_t& y, uint64_t z, uint64_t z_shoup) {
  uint64_t p2 = op.m.p * 2;
  uint64_t t = x;
  x = reduce1(y + t, p2);
  y = lazy_mul_shoup(op.m, p2 + t - y, z, z_shoup);
}

// native.rs:238-243 `reduce3`.
inline uint64_t reduce3(const NttOp& op, uint64_t a) {
  return reduce1(reduce1(a, 2 * op.m.p), op.m.p);
}

// native.rs:77-102 `forward` (constant time; the output equals `forward_vt`).
void ntt_forward(const NttOp& op, uint64_t* a) {
  size_t l = op.n >> 1;
  size_t k = 1;
  while (l > 0) {
    for (size_t s = 0; s < op.n; s += 2 * l) {
      uint64_t w = op.omegas[k];
      uint64_t ws = op.omegas_shoup[k];
      k++;
      if (l == 1) {
        butterfly(op, a[s], a[s + 1], w, ws);
        a[s] = reduce3(op, a[s]);
        a[s + 1] = reduce3(op, a[s + 1]);
      } else {
        for (size_t j = s; j < s + l; j++) butterfly(op, a[j], a[j + l], w, ws);
      }
    }
    l >>= 1;
  }
}

// native.rs:142-175 `forward_vt_lazy`: output in [0, 4p).
void ntt_forward_lazy(const NttOp& op, uint64_t* a) {
  size_t l = op.n >> 1;
  size_t m = 1;
  size_t k = 1;
  while (l > 0) {
    for (size_t i = 0; i < m; i++) {
      uint64_t w = op.omegas[k];
      uint64_t ws = op.omegas_shoup[k];
      k++;
      size_t s = 2 * i * l;
      for (size_t j = s; j < s + l; j++) butterfly(op, a[j], a[j + l], w, ws);
    }
    l >>= 1;
    m <<= 1;
  }
}

// native.rs:106-132 `backward`.
void ntt_backward(const NttOp& op, uint64_t* a) {
  size_t k = 0;
  size_t l = 1;
  while (l < op.n) {
    for (size_t s = 0; s < op.n; s += 2 * l) {
      uint64_t z = op.zetas_inv[k];
      uint64_t zs = op.zetas_inv_shoup[k];
      k++;
      for (size_t j = s; j < s + l; j++) inv_butterfly(op, a[j], a[j + l], z, zs);
    }
    l <<= 1;
  }
  for (size_t i = 0; i < op.n; i++) a[i] = mul_shoup(op.m, a[i], op.size_inv, op.size_inv_shoup);
}

// ---------------------------------------------------------------------------
// 256-bit wrapping integer, standing in for `ethnum::U256` (ethnum 1.5.2) as
// used by fhe-math/src/rns/scaler.rs:249-352. Words are little endian.
struct U256 {
  uint64_t w[4];
};

inline U256 u256_zero() { U256 r = {{0, 0, 0, 0}}; return r; }

inline U256 u256_add(const U256& a, const U256& b) {
  U256 r;
  u128 c = 0;
  for (int i = 0; i < 4; i++) {
    c += (u128)a.w[i] + b.w[i];
    r.w[i] = (uint64_t)c;
    c >>= 64;
  }
  return r;
}

inline U256 u256_sub(const U256& a, const U256& b) {
  U256 r;
  uint64_t borrow = 0;
  for (int i = 0; i < 4; i++) {
    u128 d = (u128)a.w[i] - b.w[i] - borrow;
    r.w[i] = (uint64_t)d;
    borrow = (uint64_t)(d >> 64) ? 1 : 0;
  }
  return r;
}

// Wrapping product of a 128-bit and a 128-bit value (low 256 bits are exact).
inline U256 u256_mul_128x128(u128 a, u128 b) {
  uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64);
  uint64_t b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
  U256 r = u256_zero();
  u128 p00 = (u128)a0 * b0, p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
  r.w[0] = (uint64_t)p00;
  u128 mid = (p00 >> 64) + (uint64_t)p01 + (uint64_t)p10;
  r.w[1] = (uint64_t)mid;
  u128 hi = (mid >> 64) + (p01 >> 64) + (p10 >> 64) + (uint64_t)p11;
  r.w[2] = (uint64_t)hi;
  r.w[3] = (uint64_t)(hi >> 64) + (uint64_t)(p11 >> 64);
  return r;
}

inline U256 u256_shr(const U256& a, unsigned s) {
  U256 r = u256_zero();
  if (s >= 256) return r;
  unsigned ws = s / 64, bs = s % 64;
  for (unsigned i = 0; i + ws < 4; i++) {
    uint64_t lo = a.w[i + ws] >> bs;
    uint64_t hi = (bs && i + ws + 1 < 4) ? (a.w[i + ws + 1] << (64 - bs)) : 0;
    r.w[i] = lo | hi;
  }
  return r;
}

inline U256 u256_not(const U256& a) {
  U256 r;
  for (int i = 0; i < 4; i++) r.w[i] = ~a.w[i];
  return r;
}

inline u128 u256_as_u128(const U256& a) { return ((u128)a.w[1] << 64) | a.w[0]; }

inline u128 div_ceil2(u128 x) { return (x >> 1) + (x & 1); }

}  // namespace

extern "C" {

// Layout of the scaler description shared with ora.py (`ScalerDesc`).
// Mirrors the fields of `RnsScaler` (fhe-math/src/rns/scaler.rs:51-72).
struct ora_scaler {
  uint64_t from_len;
  uint64_t to_len;
  uint64_t is_one;
  const uint64_t* to_moduli;     // [to_len][5] Modulus fields
  const uint64_t* gamma;         // [to_len]
  const uint64_t* gamma_shoup;   // [to_len]
  uint64_t theta_gamma_lo;
  uint64_t theta_gamma_hi;
  uint64_t theta_gamma_sign;
  const uint64_t* omega;         // [to_len][from_len]
  const uint64_t* omega_shoup;   // [to_len][from_len]
  const uint64_t* theta_omega_lo;    // [from_len]
  const uint64_t* theta_omega_hi;    // [from_len]
  const uint64_t* theta_omega_sign;  // [from_len]
  const uint64_t* theta_garner_lo;   // [from_len]
  const uint64_t* theta_garner_hi;   // [from_len]
  uint64_t theta_garner_shift;
};

static inline Modulus load_modulus(const uint64_t* f) {
  Modulus m;
  m.p = f[0];
  m.barrett_hi = f[1];
  m.barrett_lo = f[2];
  m.leading_zeros = f[3];
  m.supports_opt = f[4];
  return m;
}

static NttOp make_op(const uint64_t* mod, size_t n, const uint64_t* t0, const uint64_t* t1,
                     const uint64_t* t2, const uint64_t* t3, uint64_t size_inv, uint64_t size_inv_shoup) {
  NttOp op;
  op.m = load_modulus(mod);
  op.n = n;
  op.omegas = t0;
  op.omegas_shoup = t1;
  op.zetas_inv = t2;
  op.zetas_inv_shoup = t3;
  op.size_inv = size_inv;
  op.size_inv_shoup = size_inv_shoup;
  return op;
}

// ntt/native.rs:35-73 `NttOperator::new` table construction, given the root.
// powers[i] = omega^i, powers_inv[i] = omega^-(i+1), then bit-reversed.
void ora_ntt_tables(const uint64_t* mod, size_t n, uint64_t omega, uint64_t omega_inv,
                    uint64_t* omegas, uint64_t* omegas_shoup, uint64_t* zetas_inv,
                    uint64_t* zetas_inv_shoup) {
  Modulus m = load_modulus(mod);
  std::vector<uint64_t> powers(n), powers_inv(n);
  uint64_t x = 1, y = omega_inv;
  for (size_t i = 0; i < n; i++) {
    powers[i] = x;
    powers_inv[i] = y;
    x = reduce_u128(m, (u128)x * omega);
    y = reduce_u128(m, (u128)y * omega_inv);
  }
  unsigned logn = 0;
  while (((size_t)1 << logn) < n) logn++;
  for (size_t i = 0; i < n; i++) {
    size_t j = 0;
    for (unsigned b = 0; b < logn; b++)
      if (i & ((size_t)1 << b)) j |= (size_t)1 << (logn - 1 - b);
    omegas[i] = powers[j];
    zetas_inv[i] = powers_inv[j];
    omegas_shoup[i] = shoup(m, omegas[i]);
    zetas_inv_shoup[i] = shoup(m, zetas_inv[i]);
  }
}

// Runs `forward` (mode 0) or `forward_vt_lazy` (mode 1) on `rows` rows.
void ora_ntt_forward(const uint64_t* mod, size_t n, const uint64_t* omegas,
                     const uint64_t* omegas_shoup, uint64_t* a, size_t rows, int mode) {
  NttOp op = make_op(mod, n, omegas, omegas_shoup, nullptr, nullptr, 0, 0);
  for (size_t r = 0; r < rows; r++) {
    if (mode == 1) ntt_forward_lazy(op, a + r * n);
    else ntt_forward(op, a + r * n);
  }
}

void ora_ntt_backward(const uint64_t* mod, size_t n, const uint64_t* zetas_inv,
                      const uint64_t* zetas_inv_shoup, uint64_t size_inv, uint64_t size_inv_shoup,
                      uint64_t* a, size_t rows) {
  NttOp op = make_op(mod, n, nullptr, nullptr, zetas_inv, zetas_inv_shoup, size_inv, size_inv_shoup);
  for (size_t r = 0; r < rows; r++) ntt_backward(op, a + r * n);
}

// zq/mod.rs:332-344 `mul_vec`.
void ora_mul_vec(const uint64_t* mod, uint64_t* a, const uint64_t* b, size_t n) {
  Modulus m = load_modulus(mod);
  for (size_t i = 0; i < n; i++) a[i] = mul(m, a[i], b[i]);
}

// zq/mod.rs:407-416 `mul_shoup_vec`.
void ora_mul_shoup_vec(const uint64_t* mod, uint64_t* a, const uint64_t* b, const uint64_t* b_shoup,
                       size_t n) {
  Modulus m = load_modulus(mod);
  for (size_t i = 0; i < n; i++) a[i] = mul_shoup(m, a[i], b[i], b_shoup[i]);
}

// zq/mod.rs:370-374 `shoup_vec`.
void ora_shoup_vec(const uint64_t* mod, const uint64_t* a, uint64_t* out, size_t n) {
  Modulus m = load_modulus(mod);
  for (size_t i = 0; i < n; i++) out[i] = shoup(m, a[i]);
}

// zq/mod.rs:349-355 `scalar_mul_vec`.
void ora_scalar_mul_vec(const uint64_t* mod, uint64_t* a, uint64_t b, size_t n) {
  Modulus m = load_modulus(mod);
  uint64_t bs = shoup(m, b);
  for (size_t i = 0; i < n; i++) a[i] = mul_shoup(m, a[i], b, bs);
}

// zq/mod.rs:756-762 `lazy_reduce_vec`.
void ora_lazy_reduce_vec(const uint64_t* mod, uint64_t* a, size_t n) {
  Modulus m = load_modulus(mod);
  for (size_t i = 0; i < n; i++) a[i] = m.supports_opt ? lazy_reduce_opt(m, a[i]) : lazy_reduce(m, a[i]);
}

// zq/mod.rs:380-383 `reduce_vec`.
void ora_reduce_vec(const uint64_t* mod, uint64_t* a, size_t n) {
  Modulus m = load_modulus(mod);
  for (size_t i = 0; i < n; i++) a[i] = reduce(m, a[i]);
}

// One coefficient of fhe-math/src/rns/scaler.rs:249-352 `RnsScaler::scale`.
static void rns_scale_one(const ora_scaler* s, const uint64_t* rests, uint64_t* out,
                          size_t starting_index, size_t out_len) {
  const size_t L = s->from_len;
  // scaler.rs:260-269: inner product of the rests with theta_garner.
  U256 sum_theta_garner = u256_zero();
  for (size_t i = 0; i < L; i++) {
    u128 tg = ((u128)s->theta_garner_hi[i] << 64) | s->theta_garner_lo[i];
    sum_theta_garner = u256_add(sum_theta_garner, u256_mul_128x128((u128)rests[i], tg));
  }
  // scaler.rs:271-272.
  sum_theta_garner = u256_shr(sum_theta_garner, (unsigned)(s->theta_garner_shift - 1));
  u128 v = div_ceil2(u256_as_u128(sum_theta_garner));

  // scaler.rs:276-314.
  bool w_sign = false;
  u128 w = 0;
  if (!s->is_one) {
    U256 sum_theta_omega = u256_zero();
    for (size_t i = 0; i < L; i++) {
      u128 to = ((u128)s->theta_omega_hi[i] << 64) | s->theta_omega_lo[i];
      U256 product = u256_mul_128x128((u128)rests[i], to);
      if (s->theta_omega_sign[i]) sum_theta_omega = u256_sub(sum_theta_omega, product);
      else sum_theta_omega = u256_add(sum_theta_omega, product);
    }
    u128 tgam = ((u128)s->theta_gamma_hi << 64) | s->theta_gamma_lo;
    U256 v_theta_gamma = u256_mul_128x128(v, tgam);
    if (s->theta_gamma_sign) sum_theta_omega = u256_add(sum_theta_omega, v_theta_gamma);
    else sum_theta_omega = u256_sub(sum_theta_omega, v_theta_gamma);

    w_sign = (sum_theta_omega.w[3] >> 63) != 0;
    if (w_sign) {
      w = u256_as_u128(u256_shr(u256_not(sum_theta_omega), 126)) + 1;
      w /= 2;
    } else {
      w = u256_as_u128(u256_shr(sum_theta_omega, 126));
      w = div_ceil2(w);
    }
  }

  // scaler.rs:316-351.
  for (size_t i = 0; i < out_len; i++) {
    size_t j = starting_index + i;
    Modulus qi = load_modulus(s->to_moduli + 5 * j);
    u128 yi = (u128)(qi.p * 2 - lazy_mul_shoup(qi, reduce_u128(qi, v), s->gamma[j], s->gamma_shoup[j]));
    if (!s->is_one) {
      uint64_t wi = lazy_reduce_u128(qi, w);
      yi += (u128)(w_sign ? qi.p * 2 - wi : wi);
    }
    const uint64_t* om = s->omega + j * L;
    const uint64_t* oms = s->omega_shoup + j * L;
    for (size_t k = 0; k < L; k++) yi += (u128)lazy_mul_shoup(qi, rests[k], om[k], oms[k]);
    out[i] = reduce_u128(qi, yi);
  }
}

// Column loop of fhe-math/src/rq/scaler.rs:84-93: applies `RnsScaler::scale`
// to every coefficient. `in` is [from_len][n] (power basis), `out` is
// [out_len][n] and receives target moduli starting_index..starting_index+out_len.
void ora_rns_scale(const ora_scaler* s, const uint64_t* in, uint64_t* out, size_t n,
                   size_t starting_index, size_t out_len) {
  std::vector<uint64_t> col(s->from_len), res(out_len);
  for (size_t c = 0; c < n; c++) {
    for (size_t i = 0; i < s->from_len; i++) col[i] = in[i * n + c];
    rns_scale_one(s, col.data(), res.data(), starting_index, out_len);
    for (size_t i = 0; i < out_len; i++) out[i * n + c] = res[i];
  }
}

// Single coefficient column, exposed for the formula tests.
void ora_rns_scale_column(const ora_scaler* s, const uint64_t* rests, uint64_t* out,
                          size_t starting_index, size_t out_len) {
  rns_scale_one(s, rests, out, starting_index, out_len);
}

// fhe-math/src/rq/mod.rs:390-448 `Poly::switch_down` on a power-basis poly
// `a` of shape [L][n]; writes [L-1][n] into `out`. `moduli` is [L][5].
void ora_switch_down(const uint64_t* moduli, size_t L, size_t n, const uint64_t* inv_last,
                     const uint64_t* inv_last_shoup, const uint64_t* a, uint64_t* out) {
  Modulus q_last = load_modulus(moduli + 5 * (L - 1));
  uint64_t q_last_div_2 = q_last.p / 2;
  std::vector<uint64_t> last(n);
  // rq/mod.rs:417-419: add (q_last - 1)/2 to change flooring into rounding.
  for (size_t c = 0; c < n; c++) last[c] = reduce1(a[(L - 1) * n + c] + q_last_div_2, q_last.p);
  for (size_t i = 0; i + 1 < L; i++) {
    Modulus qi = load_modulus(moduli + 5 * i);
    uint64_t q_last_div_2_mod_qi = qi.p - reduce(qi, q_last_div_2);  // rq/mod.rs:427
    for (size_t c = 0; c < n; c++) {
      uint64_t tmp = lazy_reduce(qi, last[c]) + q_last_div_2_mod_qi;  // rq/mod.rs:430
      uint64_t coeff = a[i * n + c] + 3 * qi.p - tmp;                 // rq/mod.rs:434
      out[i * n + c] = mul_shoup(qi, coeff, inv_last[i], inv_last_shoup[i]);  // rq/mod.rs:437
    }
  }
}

// fhe/src/bfv/keys/key_switching_key.rs:214-241 `KeySwitchingKey::key_switch`.
// `p` is the power-basis input [count][n] (one row per ciphertext modulus);
// keys c0/c1 are [count][Lk][n] with Shoup companions; output c0/c1 [Lk][n]
// in NTT representation. `tables` holds, for each key modulus, the five
// Modulus fields followed by omegas and omegas_shoup pointers.
struct ora_ksk_limb {
  uint64_t mod[5];
  const uint64_t* omegas;
  const uint64_t* omegas_shoup;
};

void ora_key_switch(const ora_ksk_limb* limbs, size_t Lk, size_t n, const uint64_t* p, size_t count,
                    const uint64_t* c0, const uint64_t* c0_shoup, const uint64_t* c1,
                    const uint64_t* c1_shoup, uint64_t* out0, uint64_t* out1) {
  std::memset(out0, 0, sizeof(uint64_t) * Lk * n);
  std::memset(out1, 0, sizeof(uint64_t) * Lk * n);
  std::vector<uint64_t> c2i(n), prod(n);
  for (size_t i = 0; i < count; i++) {
    for (size_t j = 0; j < Lk; j++) {
      NttOp op = make_op(limbs[j].mod, n, limbs[j].omegas, limbs[j].omegas_shoup, nullptr, nullptr, 0, 0);
      // rq/mod.rs:518-540 `create_constant_ntt_polynomial_with_lazy_coefficients_and_variable_time`.
      for (size_t c = 0; c < n; c++) {
        uint64_t x = p[i * n + c];
        c2i[c] = op.m.supports_opt ? lazy_reduce_opt(op.m, x) : lazy_reduce(op.m, x);
      }
      ntt_forward_lazy(op, c2i.data());
      const size_t koff = (i * Lk + j) * n;
      // key_switching_key.rs:236-238: c0 += c2_i * c0_i; c1 += c2_i * c1_i
      // (rq/ops.rs:208-245 Shoup products, then rq/ops.rs:92-118 additions).
      for (size_t c = 0; c < n; c++) {
        uint64_t a0 = mul_shoup(op.m, c2i[c], c0[koff + c], c0_shoup[koff + c]);
        uint64_t a1 = mul_shoup(op.m, c2i[c], c1[koff + c], c1_shoup[koff + c]);
        out0[j * n + c] = reduce1(out0[j * n + c] + a0, op.m.p);
        out1[j * n + c] = reduce1(out1[j * n + c] + a1, op.m.p);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Whole products, for the timed CPU baseline: fhe/src/bfv/ops/mul.rs:158-227
// `Multiplicator::multiply` with relinearization (key at the multiplication
// level, relinearization_key.rs:71-98 without the switch-down branch), over
// independent ciphertext pairs on `threads` host threads (the reference has no
// internal parallelism; callers parallelise over ciphertexts).

// A context: moduli and NTT tables per limb (ntt/native.rs:15-73).
struct ora_ctx {
  uint64_t L, n;
  const uint64_t* moduli;  // [L][5]
  const uint64_t* const* omegas;
  const uint64_t* const* omegas_shoup;
  const uint64_t* const* zetas_inv;
  const uint64_t* const* zetas_inv_shoup;
  const uint64_t* size_inv;        // [L]
  const uint64_t* size_inv_shoup;  // [L]
};

struct ora_mult {
  ora_ctx base, mul;
  const ora_scaler* ext_lhs;
  uint64_t ncm_lhs;
  const ora_scaler* ext_rhs;
  uint64_t ncm_rhs;
  const ora_scaler* down;
  // Relinearization key (ksk context = base context): [L][L][n] values and
  // Shoup companions.
  const uint64_t* c0;
  const uint64_t* c0_shoup;
  const uint64_t* c1;
  const uint64_t* c1_shoup;
};

static NttOp ctx_op(const ora_ctx& c, size_t j) {
  return make_op(c.moduli + 5 * j, c.n, c.omegas[j], c.omegas_shoup[j], c.zetas_inv[j], c.zetas_inv_shoup[j],
                 c.size_inv[j], c.size_inv_shoup[j]);
}

// rq/scaler.rs:63-115 `Scaler::scale` of an Ntt polynomial [from.L][n] into
// [to.L][n] (Ntt): the common prefix copied, the other limbs through the
// power basis and `RnsScaler::scale`.
static void scaler_scale_ntt(const ora_scaler* s, size_t ncm, const ora_ctx& from, const ora_ctx& to,
                             const uint64_t* in, uint64_t* out, std::vector<uint64_t>& tmp) {
  const size_t n = from.n;
  std::memcpy(out, in, sizeof(uint64_t) * ncm * n);
  if (ncm >= to.L) return;
  tmp.assign(in, in + from.L * n);
  for (size_t j = 0; j < from.L; j++) ntt_backward(ctx_op(from, j), tmp.data() + j * n);
  ora_rns_scale(s, tmp.data(), out + ncm * n, n, ncm, to.L - ncm);
  for (size_t k = ncm; k < to.L; k++) ntt_forward(ctx_op(to, k), out + k * n);
}

static void multiply_one(const ora_mult* m, const uint64_t* lhs, const uint64_t* rhs, uint64_t* out,
                         std::vector<uint64_t>* buf) {
  const size_t L = m->base.L, M = m->mul.L, n = m->base.n;
  std::vector<uint64_t>& e = buf[0];    // [4][M][n]: c00, c01, c10, c11
  std::vector<uint64_t>& c = buf[1];    // [3][M][n]: the tensor
  std::vector<uint64_t>& d = buf[2];    // [3][L][n]: scaled down
  std::vector<uint64_t>& tmp = buf[3];
  std::vector<uint64_t>& ks = buf[4];   // [2][L][n]
  e.resize(4 * M * n);
  c.resize(3 * M * n);
  d.resize(3 * L * n);
  ks.resize(2 * L * n);
  // mul.rs:176-179: extend.
  for (int w = 0; w < 4; w++) {
    const bool left = w < 2;
    const uint64_t* src = (left ? lhs : rhs) + (size_t)(w & 1) * L * n;
    scaler_scale_ntt(left ? m->ext_lhs : m->ext_rhs, left ? m->ncm_lhs : m->ncm_rhs, m->base, m->mul, src,
                     e.data() + (size_t)w * M * n, tmp);
  }
  // mul.rs:182-185: c0 = c00 c10, c1 = c00 c11 + c01 c10, c2 = c01 c11.
  for (size_t j = 0; j < M; j++) {
    const Modulus q = load_modulus(m->mul.moduli + 5 * j);
    const uint64_t* c00 = e.data() + (0 * M + j) * n;
    const uint64_t* c01 = e.data() + (1 * M + j) * n;
    const uint64_t* c10 = e.data() + (2 * M + j) * n;
    const uint64_t* c11 = e.data() + (3 * M + j) * n;
    for (size_t i = 0; i < n; i++) {
      c[(0 * M + j) * n + i] = mul(q, c00[i], c10[i]);
      c[(1 * M + j) * n + i] = reduce1(mul(q, c00[i], c11[i]) + mul(q, c01[i], c10[i]), q.p);
      c[(2 * M + j) * n + i] = mul(q, c01[i], c11[i]);
    }
  }
  // mul.rs:188-190: scale down.
  for (int k = 0; k < 3; k++)
    scaler_scale_ntt(m->down, 0, m->mul, m->base, c.data() + (size_t)k * M * n, d.data() + (size_t)k * L * n, tmp);
  // mul.rs:196-210: relinearize c2.
  tmp.assign(d.data() + 2 * L * n, d.data() + 3 * L * n);
  for (size_t j = 0; j < L; j++) ntt_backward(ctx_op(m->base, j), tmp.data() + j * n);
  std::vector<ora_ksk_limb> limbs(L);
  for (size_t j = 0; j < L; j++) {
    for (int f = 0; f < 5; f++) limbs[j].mod[f] = m->base.moduli[5 * j + f];
    limbs[j].omegas = m->base.omegas[j];
    limbs[j].omegas_shoup = m->base.omegas_shoup[j];
  }
  ora_key_switch(limbs.data(), L, n, tmp.data(), L, m->c0, m->c0_shoup, m->c1, m->c1_shoup, ks.data(),
                 ks.data() + L * n);
  for (size_t part = 0; part < 2; part++)
    for (size_t j = 0; j < L; j++) {
      const uint64_t p = m->base.moduli[5 * j];
      for (size_t i = 0; i < n; i++) {
        const size_t at = (part * L + j) * n + i;
        out[at] = reduce1(d[at] + ks[at], p);
      }
    }
}

// `count` products: lhs, rhs [count][2][L][n] (Ntt) -> out [count][2][L][n].
// Pair k runs on thread k % threads.
void ora_multiply(const ora_mult* m, const uint64_t* lhs, const uint64_t* rhs, uint64_t* out, size_t count,
                  size_t threads) {
  const size_t ct = 2 * m->base.L * m->base.n;
  if (threads < 1) threads = 1;
  std::vector<std::thread> pool;
  for (size_t t = 0; t < threads; t++)
    pool.emplace_back([=] {
      std::vector<uint64_t> buf[5];
      for (size_t k = t; k < count; k += threads) multiply_one(m, lhs + k * ct, rhs + k * ct, out + k * ct, buf);
    });
  for (auto& th : pool) th.join();
}

}  // extern "C"
