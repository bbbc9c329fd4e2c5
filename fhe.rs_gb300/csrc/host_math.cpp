// Host-side number theory and precomputation (see host_math.hpp).

#include "host_math.hpp"

#include <algorithm>

#include "fheg.h"

namespace fheg {

// ---------------------------------------------------------------------------
// BigUint

BigUint::BigUint(uint64_t v) {
  if (v) {
    limbs_.push_back((uint32_t)v);
    if (v >> 32) limbs_.push_back((uint32_t)(v >> 32));
  }
}

BigUint BigUint::from_u128(u128 v) {
  BigUint r;
  while (v) {
    r.limbs_.push_back((uint32_t)v);
    v >>= 32;
  }
  return r;
}

BigUint BigUint::from_words(const uint64_t* w, size_t n) {
  BigUint r;
  for (size_t i = 0; i < n; i++) {
    r.limbs_.push_back((uint32_t)w[i]);
    r.limbs_.push_back((uint32_t)(w[i] >> 32));
  }
  r.trim();
  return r;
}

void BigUint::trim() {
  while (!limbs_.empty() && limbs_.back() == 0) limbs_.pop_back();
}

size_t BigUint::bits() const {
  if (limbs_.empty()) return 0;
  uint32_t top = limbs_.back();
  size_t b = 0;
  while (top) {
    b++;
    top >>= 1;
  }
  return (limbs_.size() - 1) * 32 + b;
}

uint64_t BigUint::low_u64() const {
  uint64_t r = 0;
  if (limbs_.size() > 0) r |= limbs_[0];
  if (limbs_.size() > 1) r |= (uint64_t)limbs_[1] << 32;
  return r;
}

u128 BigUint::low_u128() const {
  u128 r = 0;
  for (size_t i = 0; i < 4 && i < limbs_.size(); i++) r |= (u128)limbs_[i] << (32 * i);
  return r;
}

uint64_t BigUint::mod_u64(uint64_t m) const {
  u128 r = 0;
  for (size_t i = limbs_.size(); i-- > 0;) r = ((r << 32) | limbs_[i]) % m;
  return (uint64_t)r;
}

int cmp(const BigUint& a, const BigUint& b) {
  if (a.limbs_.size() != b.limbs_.size()) return a.limbs_.size() < b.limbs_.size() ? -1 : 1;
  for (size_t i = a.limbs_.size(); i-- > 0;) {
    if (a.limbs_[i] != b.limbs_[i]) return a.limbs_[i] < b.limbs_[i] ? -1 : 1;
  }
  return 0;
}

BigUint operator+(const BigUint& a, const BigUint& b) {
  BigUint r;
  size_t n = std::max(a.limbs_.size(), b.limbs_.size());
  r.limbs_.resize(n + 1);
  uint64_t c = 0;
  for (size_t i = 0; i < n; i++) {
    c += (uint64_t)(i < a.limbs_.size() ? a.limbs_[i] : 0) + (i < b.limbs_.size() ? b.limbs_[i] : 0);
    r.limbs_[i] = (uint32_t)c;
    c >>= 32;
  }
  r.limbs_[n] = (uint32_t)c;
  r.trim();
  return r;
}

BigUint operator-(const BigUint& a, const BigUint& b) {
  if (a < b) throw Error(FHEG_ERR_INTERNAL, "BigUint subtraction underflow");
  BigUint r;
  r.limbs_.resize(a.limbs_.size());
  int64_t borrow = 0;
  for (size_t i = 0; i < a.limbs_.size(); i++) {
    int64_t d = (int64_t)a.limbs_[i] - (i < b.limbs_.size() ? (int64_t)b.limbs_[i] : 0) - borrow;
    borrow = d < 0;
    if (d < 0) d += ((int64_t)1 << 32);
    r.limbs_[i] = (uint32_t)d;
  }
  r.trim();
  return r;
}

BigUint operator*(const BigUint& a, const BigUint& b) {
  BigUint r;
  if (a.is_zero() || b.is_zero()) return r;
  r.limbs_.assign(a.limbs_.size() + b.limbs_.size(), 0);
  for (size_t i = 0; i < a.limbs_.size(); i++) {
    uint64_t c = 0;
    for (size_t j = 0; j < b.limbs_.size(); j++) {
      uint64_t t = (uint64_t)a.limbs_[i] * b.limbs_[j] + r.limbs_[i + j] + c;
      r.limbs_[i + j] = (uint32_t)t;
      c = t >> 32;
    }
    size_t k = i + b.limbs_.size();
    while (c) {
      uint64_t t = (uint64_t)r.limbs_[k] + c;
      r.limbs_[k] = (uint32_t)t;
      c = t >> 32;
      k++;
    }
  }
  r.trim();
  return r;
}

BigUint operator<<(const BigUint& a, size_t s) {
  if (a.is_zero()) return a;
  BigUint r;
  size_t ws = s / 32, bs = s % 32;
  r.limbs_.assign(a.limbs_.size() + ws + 1, 0);
  for (size_t i = 0; i < a.limbs_.size(); i++) {
    uint64_t v = (uint64_t)a.limbs_[i] << bs;
    r.limbs_[i + ws] |= (uint32_t)v;
    r.limbs_[i + ws + 1] |= (uint32_t)(v >> 32);
  }
  r.trim();
  return r;
}

BigUint operator>>(const BigUint& a, size_t s) {
  BigUint r;
  size_t ws = s / 32, bs = s % 32;
  if (ws >= a.limbs_.size()) return r;
  r.limbs_.assign(a.limbs_.size() - ws, 0);
  for (size_t i = 0; i < r.limbs_.size(); i++) {
    uint64_t v = a.limbs_[i + ws];
    if (i + ws + 1 < a.limbs_.size()) v |= (uint64_t)a.limbs_[i + ws + 1] << 32;
    r.limbs_[i] = (uint32_t)(v >> bs);
  }
  r.trim();
  return r;
}

// Binary long division: the precomputation only divides numbers of a few
// thousand bits a handful of times, so the simple method is sufficient.
void BigUint::divmod(const BigUint& a, const BigUint& b, BigUint* q, BigUint* r) {
  if (b.is_zero()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "division by zero");
  if (a < b) {
    *q = BigUint();
    *r = a;
    return;
  }
  size_t shift = a.bits() - b.bits();
  BigUint rem = a;
  BigUint d = b << shift;
  BigUint quo;
  quo.limbs_.assign(shift / 32 + 1, 0);
  for (size_t i = shift + 1; i-- > 0;) {
    if (rem >= d) {
      rem = rem - d;
      quo.limbs_[i / 32] |= (uint32_t)1 << (i % 32);
    }
    d = d >> 1;
  }
  quo.trim();
  *q = quo;
  *r = rem;
}

// ---------------------------------------------------------------------------
// 64-bit modular arithmetic

uint64_t powmod(uint64_t a, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p, b = a % p;
  while (e) {
    if (e & 1) r = mulmod(r, b, p);
    b = mulmod(b, b, p);
    e >>= 1;
  }
  return r;
}

uint64_t invmod(uint64_t a, uint64_t m) {
  // Extended Euclid on signed 128-bit integers.
  __int128 t = 0, newt = 1, r = m, newr = a % m;
  while (newr != 0) {
    __int128 quotient = r / newr;
    __int128 tmp = t - quotient * newt;
    t = newt;
    newt = tmp;
    tmp = r - quotient * newr;
    r = newr;
    newr = tmp;
  }
  if (r != 1) throw Error(FHEG_ERR_INVALID_MODULUS, "value is not invertible");
  if (t < 0) t += m;
  return (uint64_t)t;
}

void barrett128(uint64_t p, uint64_t* hi, uint64_t* lo) {
  u128 all = ~(u128)0;
  u128 q = all / p;
  if (all % p == p - 1) q += 1;  // floor(2^128 / p) = floor((2^128-1)/p) (+1 if p | 2^128)
  *hi = (uint64_t)(q >> 64);
  *lo = (uint64_t)q;
}

bool is_prime(uint64_t p) {
  if (p < 2) return false;
  static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  for (uint64_t q : small) {
    if (p % q == 0) return p == q;
  }
  uint64_t d = p - 1;
  int s = 0;
  while ((d & 1) == 0) {
    d >>= 1;
    s++;
  }
  for (uint64_t a : small) {
    uint64_t x = powmod(a, d, p);
    if (x == 1 || x == p - 1) continue;
    bool composite = true;
    for (int i = 1; i < s; i++) {
      x = mulmod(x, x, p);
      if (x == p - 1) {
        composite = false;
        break;
      }
    }
    if (composite) return false;
  }
  return true;
}

static int lz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

bool supports_opt(uint64_t p) {
  // primes.rs:10-24: (2^(3s0)+1) * 2^64 < 2^(3s0) * (2^s0+1) * p with s0 = leading zeros.
  int s0 = lz64(p);
  if (s0 < 1) return false;
  BigUint middle = BigUint(1) << (size_t)(3 * s0);
  BigUint left = (middle + BigUint(1)) << 64;
  middle = middle * BigUint(((uint64_t)1 << s0) + 1);
  middle = middle * BigUint(p);
  return left < middle;
}

uint64_t generate_prime(unsigned num_bits, uint64_t modulo, uint64_t upper_bound) {
  if (num_bits < 10 || num_bits > 62) return 0;
  int lz = 64 - (int)num_bits;
  uint64_t t = upper_bound - 1;
  while (t % modulo != 1 && lz64(t) == lz) t--;
  while (lz64(t) == lz && !is_prime(t) && t >= modulo) t -= modulo;
  if (lz64(t) == lz && is_prime(t)) return t;
  return 0;
}

bool supports_ntt(uint64_t p, size_t n) {
  if (n < 8 || (n & (n - 1))) return false;
  return p % ((uint64_t)n << 1) == 1 && is_prime(p);
}

// ---------------------------------------------------------------------------
// Default NTT root. `NttOperator::primitive_root` draws candidates from
// `ChaCha8Rng::seed_from_u64(0)` with `random_range(0..p)`. The generator
// below follows the published algorithms of those third-party crates:
// rand_core 0.9.3 seeds from a u64 with a PCG32 stream, rand_chacha 0.9.0 is
// the ChaCha block function (8 rounds, 64-bit block counter, 64-bit stream id
// zero) whose output words are consumed in order, two per u64 (low first),
// and rand 0.9.2 samples a range with Canon's method.

namespace {

inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

struct ChaCha8 {
  uint32_t key[8];
  uint64_t counter = 0;
  uint32_t buf[16];
  int idx = 16;

  explicit ChaCha8(uint64_t state) {
    const uint64_t mul = 6364136223846793005ULL, inc = 11634580027462260723ULL;
    for (int i = 0; i < 8; i++) {
      state = state * mul + inc;
      uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
      uint32_t rot = (uint32_t)(state >> 59);
      key[i] = (xorshifted >> rot) | (xorshifted << ((32 - rot) & 31));
    }
  }

  void refill() {
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    for (int i = 0; i < 8; i++) st[4 + i] = key[i];
    st[12] = (uint32_t)counter;
    st[13] = (uint32_t)(counter >> 32);
    st[14] = 0;
    st[15] = 0;
    uint32_t x[16];
    for (int i = 0; i < 16; i++) x[i] = st[i];
    auto qr = [&](int a, int b, int c, int d) {
      x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);
      x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);
      x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);
      x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
    };
    for (int r = 0; r < 4; r++) {
      qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15);
      qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14);
    }
    for (int i = 0; i < 16; i++) buf[i] = x[i] + st[i];
    counter++;
    idx = 0;
  }

  uint32_t next_u32() {
    if (idx >= 16) refill();
    return buf[idx++];
  }

  uint64_t next_u64() {
    uint64_t lo = next_u32();
    uint64_t hi = next_u32();
    return lo | (hi << 32);
  }

  uint64_t range(uint64_t low, uint64_t high) {
    uint64_t range = high - low;  // (high - 1) - low + 1
    if (range == 0) return next_u64();
    u128 prod = (u128)next_u64() * range;
    uint64_t result = (uint64_t)(prod >> 64), lo_order = (uint64_t)prod;
    if (lo_order > (uint64_t)(0 - range)) {
      uint64_t new_hi = (uint64_t)(((u128)next_u64() * range) >> 64);
      if ((u128)lo_order + new_hi > (u128)UINT64_MAX) result += 1;
    }
    return low + result;
  }
};

}  // namespace

uint64_t default_ntt_root(uint64_t p, size_t n) {
  if (!supports_ntt(p, n)) throw Error(FHEG_ERR_NTT_UNSUPPORTED, "Impossible to construct a Ntt operator");
  uint64_t lambda = (p - 1) / (2 * (uint64_t)n);
  ChaCha8 rng(0);
  for (int i = 0; i < 100; i++) {
    uint64_t root = rng.range(0, p);
    root = powmod(root, lambda, p);
    // native.rs:341-348 `is_primitive_root`
    if (powmod(root, 2 * (uint64_t)n, p) == 1 && powmod(root, (uint64_t)n, p) != 1) return root;
  }
  throw Error(FHEG_ERR_NTT_UNSUPPORTED, "Couldn't find primitive root");
}

NttTablesHost make_ntt_tables(uint64_t p, size_t n, uint64_t root) {
  if (p < 2 || (p >> 62) != 0) throw Error(FHEG_ERR_INVALID_MODULUS, "InvalidModulus");
  if (!supports_ntt(p, n)) throw Error(FHEG_ERR_NTT_UNSUPPORTED, "Impossible to construct a Ntt operator");
  if (root == 0) root = default_ntt_root(p, n);
  if (powmod(root, 2 * (uint64_t)n, p) != 1 || powmod(root, (uint64_t)n, p) == 1)
    throw Error(FHEG_ERR_INVALID_ARGUMENT, "the injected root is not a primitive 2n-th root of unity");
  NttTablesHost t;
  t.p = p;
  t.n = n;
  t.root = root;
  t.size_inv = invmod(n % p, p);
  t.size_inv_shoup = shoup(t.size_inv, p);
  uint64_t root_inv = invmod(root, p);
  std::vector<uint64_t> powers(n), powers_inv(n);
  uint64_t x = 1, y = root_inv;
  for (size_t i = 0; i < n; i++) {
    powers[i] = x;
    powers_inv[i] = y;
    x = mulmod(x, root, p);
    y = mulmod(y, root_inv, p);
  }
  int logn = 0;
  while (((size_t)1 << logn) < n) logn++;
  t.omegas.resize(n);
  t.omegas_shoup.resize(n);
  t.zetas_inv.resize(n);
  t.zetas_inv_shoup.resize(n);
  for (size_t i = 0; i < n; i++) {
    size_t j = 0;
    for (int b = 0; b < logn; b++)
      if (i & ((size_t)1 << b)) j |= (size_t)1 << (logn - 1 - b);
    t.omegas[i] = powers[j];
    t.zetas_inv[i] = powers_inv[j];
    t.omegas_shoup[i] = shoup(t.omegas[i], p);
    t.zetas_inv_shoup[i] = shoup(t.zetas_inv[i], p);
  }
  return t;
}

// ---------------------------------------------------------------------------
// RNS

RnsContextHost::RnsContextHost(const std::vector<uint64_t>& m) : moduli(m) {
  if (m.empty()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The list of moduli is empty");
  product = BigUint(1);
  for (size_t i = 0; i < m.size(); i++) {
    for (size_t j = 0; j < m.size(); j++) {
      if (i != j) {
        uint64_t a = m[i], b = m[j];
        while (b) {
          uint64_t r = a % b;
          a = b;
          b = r;
        }
        if (a != 1) throw Error(FHEG_ERR_INVALID_ARGUMENT, "The moduli are not coprime");
      }
    }
    product = product * BigUint(m[i]);
  }
  for (uint64_t q : m) {
    BigUint q_star = product / BigUint(q);
    uint64_t q_tilde = invmod(q_star.mod_u64(q), q);
    garner.push_back(q_star * BigUint(q_tilde));
  }
}

namespace {

struct ProjTheta {
  std::vector<uint64_t> projected;
  uint64_t lo, hi;
  bool sign;
};

// rns/scaler.rs:183-229 `extract_projection_and_theta`.
ProjTheta extract_projection_and_theta(const RnsContextHost& ctx, const BigUint& input, const BigUint& num,
                                       const BigUint& den, bool round_up) {
  ProjTheta r;
  BigUint prod = num * input;
  BigUint gamma = (prod + (den >> 1)) / den;
  for (uint64_t q : ctx.moduli) r.projected.push_back(gamma.mod_u64(q));
  BigUint theta = prod % den;
  r.sign = false;
  BigUint half = den >> 1;
  if (den > BigUint(1)) {
    if (den.is_odd()) {
      if (theta > half) {
        r.sign = true;
        theta = den - theta;
      }
    } else if (theta >= half) {
      r.sign = true;
      theta = den - theta;
    }
  }
  BigUint one(1);
  bool ceil = round_up ? !r.sign : r.sign;
  if (ceil) theta = ((theta << 127) + den - one) / den;
  else theta = (theta << 127) / den;
  u128 t = theta.low_u128();
  r.lo = (uint64_t)t;
  r.hi = (uint64_t)(t >> 64);
  return r;
}

size_t ilog2_next_pow2(u128 x) {
  // ilog2 of the smallest power of two >= x (x >= 1).
  size_t k = 0;
  while (((u128)1 << k) < x) k++;
  return k;
}

}  // namespace

RnsScalerHost make_rns_scaler(const RnsContextHost& from, const RnsContextHost& to, const BigUint& num,
                              const BigUint& den) {
  if (den.is_zero()) throw Error(FHEG_ERR_INVALID_ARGUMENT, "ScalingFactor denominator is zero");
  RnsScalerHost s;
  s.from_len = from.moduli.size();
  s.to_len = to.moduli.size();
  s.is_one = (num == den);
  // scaler.rs:85-95: gamma = round(num * from.product / den).
  ProjTheta g = extract_projection_and_theta(to, from.product, num, den, false);
  s.gamma = g.projected;
  s.theta_gamma_lo = g.lo;
  s.theta_gamma_hi = g.hi;
  s.theta_gamma_sign = g.sign;
  for (size_t j = 0; j < s.to_len; j++) s.gamma_shoup.push_back(shoup(s.gamma[j], to.moduli[j]));
  // scaler.rs:97-126: omega_i = round(from.garner_i * num / den).
  s.omega.assign(s.to_len * s.from_len, 0);
  s.omega_shoup.assign(s.to_len * s.from_len, 0);
  for (size_t i = 0; i < s.from_len; i++) {
    ProjTheta o = extract_projection_and_theta(to, from.garner[i], num, den, true);
    s.theta_omega_lo.push_back(o.lo);
    s.theta_omega_hi.push_back(o.hi);
    s.theta_omega_sign.push_back(o.sign ? 1 : 0);
    for (size_t j = 0; j < s.to_len; j++) {
      uint64_t v = o.projected[j] % to.moduli[j];
      s.omega[j * s.from_len + i] = v;
      s.omega_shoup[j * s.from_len + i] = shoup(v, to.moduli[j]);
    }
  }
  // scaler.rs:130-142.
  uint64_t shift = 127;
  for (uint64_t q : from.moduli) {
    uint64_t cand = 191 - ilog2_next_pow2((u128)q * (u128)from.moduli.size());
    shift = std::min(shift, cand);
  }
  s.theta_garner_shift = shift;
  // scaler.rs:145-155.
  BigUint half = from.product >> 1;
  for (size_t i = 0; i < s.from_len; i++) {
    BigUint theta = ((from.garner[i] << shift) + half) / from.product;
    u128 t = theta.low_u128();
    s.theta_garner_lo.push_back((uint64_t)t);
    s.theta_garner_hi.push_back((uint64_t)(t >> 64));
  }
  return s;
}

}  // namespace fheg
