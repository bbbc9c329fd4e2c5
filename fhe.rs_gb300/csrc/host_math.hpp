// Host-side number theory and precomputation for the GB300 RNS-BFV library.
//
// Everything here runs once per context / scaler / key on the host; the
// results are uploaded to the device. The algorithms follow fhe-math
// (paths relative to the fhe.rs repository root).
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace fheg {

typedef unsigned __int128 u128;

// Library error carrying one of the fheg_status codes.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

// Arbitrary precision unsigned integer (little-endian 32-bit limbs), used for
// the big-integer precomputation of fhe-math/src/rns (num-bigint there).
class BigUint {
 public:
  BigUint() {}
  explicit BigUint(uint64_t v);
  static BigUint from_u128(u128 v);
  static BigUint from_words(const uint64_t* w, size_t n);

  bool is_zero() const { return limbs_.empty(); }
  size_t bits() const;
  uint64_t low_u64() const;
  u128 low_u128() const;
  uint64_t mod_u64(uint64_t m) const;
  bool is_odd() const { return !limbs_.empty() && (limbs_[0] & 1); }

  friend int cmp(const BigUint& a, const BigUint& b);
  friend bool operator==(const BigUint& a, const BigUint& b) { return cmp(a, b) == 0; }
  friend bool operator!=(const BigUint& a, const BigUint& b) { return cmp(a, b) != 0; }
  friend bool operator<(const BigUint& a, const BigUint& b) { return cmp(a, b) < 0; }
  friend bool operator>(const BigUint& a, const BigUint& b) { return cmp(a, b) > 0; }
  friend bool operator>=(const BigUint& a, const BigUint& b) { return cmp(a, b) >= 0; }
  friend bool operator<=(const BigUint& a, const BigUint& b) { return cmp(a, b) <= 0; }

  friend BigUint operator+(const BigUint& a, const BigUint& b);
  friend BigUint operator-(const BigUint& a, const BigUint& b);  // requires a >= b
  friend BigUint operator*(const BigUint& a, const BigUint& b);
  friend BigUint operator<<(const BigUint& a, size_t s);
  friend BigUint operator>>(const BigUint& a, size_t s);
  // Quotient and remainder; throws on division by zero.
  static void divmod(const BigUint& a, const BigUint& b, BigUint* q, BigUint* r);
  friend BigUint operator/(const BigUint& a, const BigUint& b) {
    BigUint q, r;
    divmod(a, b, &q, &r);
    return q;
  }
  friend BigUint operator%(const BigUint& a, const BigUint& b) {
    BigUint q, r;
    divmod(a, b, &q, &r);
    return r;
  }

 private:
  void trim();
  std::vector<uint32_t> limbs_;
};

// ---- 64-bit modular helpers (fhe-math/src/zq/mod.rs) ----
inline uint64_t mulmod(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)((u128)a * b % p); }
uint64_t powmod(uint64_t a, uint64_t e, uint64_t p);
// Inverse of a modulo m for coprime a, m (extended Euclid); throws otherwise.
uint64_t invmod(uint64_t a, uint64_t m);
// zq/mod.rs:195-199 `shoup`: floor(a * 2^64 / p).
inline uint64_t shoup(uint64_t a, uint64_t p) { return (uint64_t)(((u128)a << 64) / p); }
// floor(2^128 / p) split into (hi, lo): the Barrett constant of zq/mod.rs:83-98.
void barrett128(uint64_t p, uint64_t* hi, uint64_t* lo);

// fhe-util/src/lib.rs:16-18 `is_prime` (deterministic for u64).
bool is_prime(uint64_t p);
// fhe-math/src/zq/primes.rs:10-24 `supports_opt`.
bool supports_opt(uint64_t p);
// fhe-math/src/zq/primes.rs:30-59 `generate_prime`; returns 0 when none.
uint64_t generate_prime(unsigned num_bits, uint64_t modulo, uint64_t upper_bound);
// fhe-math/src/ntt/mod.rs:19-23 `supports_ntt`.
bool supports_ntt(uint64_t p, size_t n);

// fhe-math/src/ntt/native.rs:320-336 `primitive_root`: the default root.
uint64_t default_ntt_root(uint64_t p, size_t n);

// fhe-math/src/ntt/native.rs:35-73 `NttOperator::new`: the four twiddle
// tables (bit-reversed powers of omega and of omega^-1 shifted by one) and
// the Shoup companions, plus size_inv and its Shoup companion.
struct NttTablesHost {
  uint64_t p = 0;
  size_t n = 0;
  uint64_t root = 0;
  std::vector<uint64_t> omegas, omegas_shoup, zetas_inv, zetas_inv_shoup;
  uint64_t size_inv = 0, size_inv_shoup = 0;
};
NttTablesHost make_ntt_tables(uint64_t p, size_t n, uint64_t root /* 0 = default */);

// fhe-math/src/rns/mod.rs:52-113 `RnsContext::new` (product and Garner terms).
struct RnsContextHost {
  std::vector<uint64_t> moduli;
  BigUint product;
  std::vector<BigUint> garner;
  explicit RnsContextHost(const std::vector<uint64_t>& moduli);
};

// fhe-math/src/rns/scaler.rs:51-175 `RnsScaler::new`.
struct RnsScalerHost {
  size_t from_len = 0, to_len = 0;
  bool is_one = false;
  uint64_t theta_garner_shift = 0;
  uint64_t theta_gamma_lo = 0, theta_gamma_hi = 0;
  bool theta_gamma_sign = false;
  std::vector<uint64_t> gamma, gamma_shoup;           // [to]
  std::vector<uint64_t> omega, omega_shoup;           // [to][from]
  std::vector<uint64_t> theta_omega_lo, theta_omega_hi;  // [from]
  std::vector<uint8_t> theta_omega_sign;                 // [from]
  std::vector<uint64_t> theta_garner_lo, theta_garner_hi;  // [from]
};
RnsScalerHost make_rns_scaler(const RnsContextHost& from, const RnsContextHost& to, const BigUint& num,
                              const BigUint& den);

}  // namespace fheg
