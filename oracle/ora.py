"""CPU oracle for the fhe.rs RNS-BFV ciphertext hot path.

TEST INFRASTRUCTURE ONLY. Only `tests/`, `__graft_entry__.smoke()` and the CPU
baseline leg of `bench.py` import this module; the GPU library never does.

The oracle restates the reference crates `fhe-math` and `fhe` of
stevennevins/fhe.rs. Constants that need arbitrary precision are computed here
with Python integers, following the reference line by line. The hot loops
(NTT butterflies, RNS scaling, switch-down, key switching) run in
`oracle/oracle.cpp`, which restates the corresponding Rust loops. Every
function cites the reference file:line it follows; paths are relative to the
reference repository root.

Parity pins:
  * `generate_prime` reproduces the NFLlib 62-bit prime list that
    fhe-math/src/zq/primes.rs:67-102 pins (the only literal golden vector of the
    reference for this path).
  * The scaler, switch-down, substitution and NTT loops are checked against the
    reference's own exact-formula tests restated in tests/test_oracle_*.py.
  * The NTT root is chosen by restating the published algorithms of the
    third-party crates rand_core 0.9.3 (`seed_from_u64`, PCG32 expansion),
    rand_chacha 0.9.0 (ChaCha with 8 rounds) and rand 0.9.2 (`random_range`,
    Canon's single-sample method). No reference test pins the resulting root,
    so NTT-domain values are "parity unpinned" against a real fhe.rs run.
"""

from __future__ import annotations

import ctypes
import hashlib
import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

U64P = ctypes.POINTER(ctypes.c_uint64)
M64 = (1 << 64) - 1


def lib():
    """Loads the compiled oracle loops (built by oracle/build.py)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            from . import build as _build  # type: ignore

            _build.build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


class OraScaler(ctypes.Structure):
    _fields_ = [
        ("from_len", ctypes.c_uint64),
        ("to_len", ctypes.c_uint64),
        ("is_one", ctypes.c_uint64),
        ("to_moduli", U64P),
        ("gamma", U64P),
        ("gamma_shoup", U64P),
        ("theta_gamma_lo", ctypes.c_uint64),
        ("theta_gamma_hi", ctypes.c_uint64),
        ("theta_gamma_sign", ctypes.c_uint64),
        ("omega", U64P),
        ("omega_shoup", U64P),
        ("theta_omega_lo", U64P),
        ("theta_omega_hi", U64P),
        ("theta_omega_sign", U64P),
        ("theta_garner_lo", U64P),
        ("theta_garner_hi", U64P),
        ("theta_garner_shift", ctypes.c_uint64),
    ]


class OraKskLimb(ctypes.Structure):
    _fields_ = [("mod", ctypes.c_uint64 * 5), ("omegas", U64P), ("omegas_shoup", U64P)]


class OraCtx(ctypes.Structure):
    _fields_ = [("L", ctypes.c_uint64), ("n", ctypes.c_uint64), ("moduli", U64P),
                ("omegas", ctypes.POINTER(U64P)), ("omegas_shoup", ctypes.POINTER(U64P)),
                ("zetas_inv", ctypes.POINTER(U64P)), ("zetas_inv_shoup", ctypes.POINTER(U64P)),
                ("size_inv", U64P), ("size_inv_shoup", U64P)]


class OraMult(ctypes.Structure):
    _fields_ = [("base", OraCtx), ("mul", OraCtx), ("ext_lhs", ctypes.POINTER(OraScaler)), ("ncm_lhs", ctypes.c_uint64),
                ("ext_rhs", ctypes.POINTER(OraScaler)), ("ncm_rhs", ctypes.c_uint64),
                ("down", ctypes.POINTER(OraScaler)), ("c0", U64P), ("c0_shoup", U64P), ("c1", U64P),
                ("c1_shoup", U64P)]


def _declare(L):
    sz = ctypes.c_size_t
    L.ora_ntt_tables.argtypes = [U64P, sz, ctypes.c_uint64, ctypes.c_uint64, U64P, U64P, U64P, U64P]
    L.ora_ntt_forward.argtypes = [U64P, sz, U64P, U64P, U64P, sz, ctypes.c_int]
    L.ora_ntt_backward.argtypes = [U64P, sz, U64P, U64P, ctypes.c_uint64, ctypes.c_uint64, U64P, sz]
    L.ora_mul_vec.argtypes = [U64P, U64P, U64P, sz]
    L.ora_mul_shoup_vec.argtypes = [U64P, U64P, U64P, U64P, sz]
    L.ora_shoup_vec.argtypes = [U64P, U64P, U64P, sz]
    L.ora_scalar_mul_vec.argtypes = [U64P, U64P, ctypes.c_uint64, sz]
    L.ora_lazy_reduce_vec.argtypes = [U64P, U64P, sz]
    L.ora_reduce_vec.argtypes = [U64P, U64P, sz]
    L.ora_rns_scale.argtypes = [ctypes.POINTER(OraScaler), U64P, U64P, sz, sz, sz]
    L.ora_rns_scale_column.argtypes = [ctypes.POINTER(OraScaler), U64P, U64P, sz, sz]
    L.ora_switch_down.argtypes = [U64P, sz, sz, U64P, U64P, U64P, U64P]
    L.ora_key_switch.argtypes = [ctypes.POINTER(OraKskLimb), sz, sz, U64P, sz, U64P, U64P, U64P, U64P,
                                 U64P, U64P]
    L.ora_multiply.argtypes = [ctypes.POINTER(OraMult), U64P, U64P, U64P, sz, sz]


def _p(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(U64P)


def _u64(values) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(values, dtype=np.uint64))


# ---------------------------------------------------------------------------
# fhe-util: primality.


def is_prime(p: int) -> bool:
    """fhe-util/src/lib.rs:16-18 `is_prime` (exact for u64).

    Restated as a deterministic Miller-Rabin test; the bases below are exact
    for every integer below 3.3e24.
    """
    if p < 2:
        return False
    small = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)
    for q in small:
        if p % q == 0:
            return p == q
    d, s = p - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in small:
        x = pow(a, d, p)
        if x in (1, p - 1):
            continue
        for _ in range(s - 1):
            x = x * x % p
            if x == p - 1:
                break
        else:
            return False
    return True


# ---------------------------------------------------------------------------
# fhe-math/src/zq/primes.rs


def leading_zeros(x: int) -> int:
    return 64 - x.bit_length()


def supports_opt(p: int) -> bool:
    """primes.rs:10-24 `supports_opt` (Equation (1) of the NFLlib paper)."""
    lz = leading_zeros(p)
    if lz < 1:
        return False
    middle = 1 << (3 * lz)
    left_side = (middle + 1) << 64
    middle *= (1 << lz) + 1
    middle *= p
    return left_side < middle


def generate_prime(num_bits: int, modulo: int, upper_bound: int) -> Optional[int]:
    """primes.rs:30-59 `generate_prime`."""
    if not (10 <= num_bits <= 62):
        return None
    lz = 64 - num_bits
    t = upper_bound - 1
    while t % modulo != 1 and leading_zeros(t) == lz:
        t -= 1
    while leading_zeros(t) == lz and not is_prime(t) and t >= modulo:
        t -= modulo
    if leading_zeros(t) == lz and is_prime(t):
        return t
    return None


def supports_ntt(p: int, n: int) -> bool:
    """ntt/mod.rs:19-23 `supports_ntt`."""
    assert n >= 8 and n & (n - 1) == 0
    return p % (n << 1) == 1 and is_prime(p)


# ---------------------------------------------------------------------------
# Third-party RNG algorithms used by `NttOperator::primitive_root`
# (ntt/native.rs:320-336): restated from their published descriptions.


def _rotl32(x: int, r: int) -> int:
    return ((x << r) | (x >> (32 - r))) & 0xFFFFFFFF


class ChaChaRng:
    """ChaCha keystream generator with a 64-bit block counter and a 64-bit
    stream id (the rand_chacha 0.9.0 layout), 8 rounds for ChaCha8Rng.

    Words are produced block after block; `next_u64` joins two consecutive
    words, low word first (rand_core 0.9.3 `BlockRng::next_u64`).
    """

    def __init__(self, key_words: Sequence[int], rounds: int = 8):
        assert len(key_words) == 8
        self.key = [w & 0xFFFFFFFF for w in key_words]
        self.rounds = rounds
        self.counter = 0
        self.buf: List[int] = []
        self.idx = 0

    @staticmethod
    def seed_from_u64(state: int, rounds: int = 8) -> "ChaChaRng":
        """rand_core 0.9.3 `SeedableRng::seed_from_u64`: PCG32 fills the seed."""
        mul, inc = 6364136223846793005, 11634580027462260723
        words = []
        for _ in range(8):
            state = (state * mul + inc) & M64
            xorshifted = (((state >> 18) ^ state) >> 27) & 0xFFFFFFFF
            rot = state >> 59
            words.append(((xorshifted >> rot) | (xorshifted << ((32 - rot) & 31))) & 0xFFFFFFFF)
        return ChaChaRng(words, rounds)

    def _block(self) -> List[int]:
        c = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574]
        st = c + self.key + [self.counter & 0xFFFFFFFF, self.counter >> 32, 0, 0]
        x = list(st)

        def qr(a, b, cc, d):
            x[a] = (x[a] + x[b]) & 0xFFFFFFFF
            x[d] = _rotl32(x[d] ^ x[a], 16)
            x[cc] = (x[cc] + x[d]) & 0xFFFFFFFF
            x[b] = _rotl32(x[b] ^ x[cc], 12)
            x[a] = (x[a] + x[b]) & 0xFFFFFFFF
            x[d] = _rotl32(x[d] ^ x[a], 8)
            x[cc] = (x[cc] + x[d]) & 0xFFFFFFFF
            x[b] = _rotl32(x[b] ^ x[cc], 7)

        for _ in range(self.rounds // 2):
            qr(0, 4, 8, 12)
            qr(1, 5, 9, 13)
            qr(2, 6, 10, 14)
            qr(3, 7, 11, 15)
            qr(0, 5, 10, 15)
            qr(1, 6, 11, 12)
            qr(2, 7, 8, 13)
            qr(3, 4, 9, 14)
        self.counter = (self.counter + 1) & M64
        return [(x[i] + st[i]) & 0xFFFFFFFF for i in range(16)]

    def next_u32(self) -> int:
        if self.idx >= len(self.buf):
            self.buf = self._block()
            self.idx = 0
        w = self.buf[self.idx]
        self.idx += 1
        return w

    def next_u64(self) -> int:
        lo = self.next_u32()
        hi = self.next_u32()
        return lo | (hi << 32)

    @staticmethod
    def from_seed(seed: bytes, rounds: int = 8) -> "ChaChaRng":
        """rand_chacha 0.9.0 `SeedableRng::from_seed`: the 32 seed bytes are
        the key as little-endian words; counter and stream start at zero."""
        assert len(seed) == 32
        return ChaChaRng([int.from_bytes(seed[4 * i:4 * i + 4], "little") for i in range(8)], rounds)

    def fill_bytes(self, n: int) -> bytes:
        """rand_core 0.9.3 `BlockRng::fill_bytes` (`Rng::fill` of a byte
        array): whole words, little-endian; the rest of a last partial word is
        dropped."""
        out = bytearray()
        while len(out) < n:
            out += self.next_u32().to_bytes(4, "little")
        return bytes(out[:n])

    def random_range_u64(self, low: int, high: int) -> int:
        """rand 0.9.2 `random_range(low..high)` for u64 (Canon's method with
        one extra sample to reduce bias)."""
        hi_incl = high - 1
        rng_range = (hi_incl - low + 1) & M64
        if rng_range == 0:
            return self.next_u64()
        prod = self.next_u64() * rng_range
        result, lo_order = prod >> 64, prod & M64
        if lo_order > ((-rng_range) & M64):
            new_hi = (self.next_u64() * rng_range) >> 64
            if lo_order + new_hi > M64:
                result += 1
        return (low + result) & M64


def chacha_blocks(key_words: Sequence[int], counters: np.ndarray, rounds: int = 8, stream: int = 0) -> np.ndarray:
    """The block function of `ChaChaRng._block`, vectorised over block
    counters: [len(counters), 16] uint32 keystream words."""
    ctr = np.asarray(counters, dtype=np.uint64)
    n = ctr.shape[0]
    st = np.zeros((16, n), dtype=np.uint32)
    st[0:4] = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)[:, None]
    st[4:12] = np.array([w & 0xFFFFFFFF for w in key_words], dtype=np.uint32)[:, None]
    st[12] = (ctr & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    st[13] = (ctr >> np.uint64(32)).astype(np.uint32)
    st[14] = stream & 0xFFFFFFFF
    st[15] = (stream >> 32) & 0xFFFFFFFF
    x = st.copy()

    def rotl(v, r):
        return (v << np.uint32(r)) | (v >> np.uint32(32 - r))

    def qr(a, b, c, d):
        x[a] += x[b]
        x[d] = rotl(x[d] ^ x[a], 16)
        x[c] += x[d]
        x[b] = rotl(x[b] ^ x[c], 12)
        x[a] += x[b]
        x[d] = rotl(x[d] ^ x[a], 8)
        x[c] += x[d]
        x[b] = rotl(x[b] ^ x[c], 7)

    for _ in range(rounds // 2):
        qr(0, 4, 8, 12)
        qr(1, 5, 9, 13)
        qr(2, 6, 10, 14)
        qr(3, 7, 11, 15)
        qr(0, 5, 10, 15)
        qr(1, 6, 11, 12)
        qr(2, 7, 8, 13)
        qr(3, 4, 9, 14)
    return (x + st).T.copy()


def chacha_u64_draws(key_words: Sequence[int], first: int, count: int, rounds: int = 8) -> np.ndarray:
    """Draws first .. first+count-1 of `next_u64` on a fresh generator: draw
    k joins words 2k (low) and 2k+1 (high) of the keystream."""
    b0, b1 = first // 8, (first + count + 7) // 8
    w = chacha_blocks(key_words, np.arange(b0, b1, dtype=np.uint64), rounds).reshape(-1).astype(np.uint64)
    d = w[0::2] | (w[1::2] << np.uint64(32))
    return d[first - 8 * b0:first - 8 * b0 + count]


def uniform_u64_threshold(q: int) -> int:
    """rand 0.9.2 `UniformInt<u64>` for the range [0, q): a draw x gives the
    high word of x q unless the low word is below (2^64 - q) mod q, in which
    case it is redrawn (Lemire's widening multiply with rejection). The
    rejection rule is restated from the published method; no reference test
    pins it."""
    return ((1 << 64) - q) % q


def random_from_seed(ctx: "Context", seed: bytes) -> np.ndarray:
    """rq/mod.rs:239-257 `Poly::random_from_seed`: SHA-256 of the seed is the
    key of a ChaCha8 generator, and each limb takes `degree` samples of
    Uniform[0, q_j) in turn (`Modulus::random_vec`, zq/mod.rs:765-767).
    Returns the [L][N] coefficients (used as is in every representation)."""
    digest = hashlib.sha256(bytes(seed)).digest()
    key = [int.from_bytes(digest[4 * i:4 * i + 4], "little") for i in range(8)]
    n = ctx.degree
    out = np.zeros((len(ctx.moduli), n), dtype=np.uint64)
    pos = 0
    for j, q in enumerate(ctx.moduli):
        thresh = uniform_u64_threshold(q)
        vals: List[int] = []
        while len(vals) < n:
            want = n - len(vals)
            draws = chacha_u64_draws(key, pos, want + 8).astype(object)
            prod = draws * q
            for k in range(want + 8):
                if int(prod[k]) & M64 >= thresh:
                    vals.append(int(prod[k]) >> 64)
                    if len(vals) == n:
                        pos += k + 1
                        break
            else:
                pos += want + 8
        out[j] = np.array(vals, dtype=np.uint64)
    return out


def ksk_c1_seeds(seed: bytes, size: int) -> List[bytes]:
    """key_switching_key.rs:108-123 `generate_c1`: seed i of c1[i] is the
    next 32 bytes of a ChaCha8 generator keyed with the key's seed."""
    rng = ChaChaRng.from_seed(bytes(seed))
    return [rng.fill_bytes(32) for _ in range(size)]


# ---------------------------------------------------------------------------
# fhe-math/src/zq/mod.rs


class Modulus:
    """zq/mod.rs:31-98 `Modulus` (constants only; arithmetic runs in C)."""

    def __init__(self, p: int):
        if p < 2 or (p >> 62) != 0:
            raise ValueError(f"InvalidModulus({p})")
        self.p = p
        barrett = (1 << 128) // p
        self.barrett_hi = barrett >> 64
        self.barrett_lo = barrett & M64
        self.leading_zeros = leading_zeros(p)
        self.supports_opt = supports_opt(p)
        self.fields = _u64([p, self.barrett_hi, self.barrett_lo, self.leading_zeros, int(self.supports_opt)])

    def __eq__(self, other):
        return isinstance(other, Modulus) and other.p == self.p

    def __hash__(self):
        return hash(self.p)

    # scalar helpers (zq/mod.rs:556-590)
    def pow(self, a: int, n: int) -> int:
        return pow(a, n, self.p)

    def inv(self, a: int) -> Optional[int]:
        if not is_prime(self.p) or a % self.p == 0:
            return None
        return pow(a, self.p - 2, self.p)

    def shoup(self, a: int) -> int:
        return (a << 64) // self.p

    # vector helpers (in place on numpy rows)
    def mul_vec(self, a: np.ndarray, b: np.ndarray):
        lib().ora_mul_vec(_p(self.fields), _p(a), _p(b), a.size)

    def mul_shoup_vec(self, a: np.ndarray, b: np.ndarray, b_shoup: np.ndarray):
        lib().ora_mul_shoup_vec(_p(self.fields), _p(a), _p(b), _p(b_shoup), a.size)

    def shoup_vec(self, a: np.ndarray) -> np.ndarray:
        out = np.empty_like(a)
        lib().ora_shoup_vec(_p(self.fields), _p(a), _p(out), a.size)
        return out

    def scalar_mul_vec(self, a: np.ndarray, b: int):
        lib().ora_scalar_mul_vec(_p(self.fields), _p(a), b % self.p, a.size)

    def reduce_vec(self, a: np.ndarray):
        lib().ora_reduce_vec(_p(self.fields), _p(a), a.size)

    def lazy_reduce_vec(self, a: np.ndarray):
        lib().ora_lazy_reduce_vec(_p(self.fields), _p(a), a.size)

    def add_vec(self, a: np.ndarray, b: np.ndarray):
        """zq/mod.rs:240-280 (operands < p < 2^62, so the sum fits in u64)."""
        s = a + b
        np.subtract(s, np.uint64(self.p), out=s, where=s >= np.uint64(self.p))
        a[...] = s

    def sub_vec(self, a: np.ndarray, b: np.ndarray):
        s = a + (np.uint64(self.p) - b)
        np.subtract(s, np.uint64(self.p), out=s, where=s >= np.uint64(self.p))
        a[...] = s

    def neg_vec(self, a: np.ndarray):
        s = np.uint64(self.p) - a
        s[s == np.uint64(self.p)] = 0
        a[...] = s

    def reduce_vec_i64(self, a: np.ndarray) -> np.ndarray:
        """zq/mod.rs:479-499 `reduce_vec_i64`."""
        return _u64(np.mod(a.astype(object), self.p).astype(np.uint64))


# ---------------------------------------------------------------------------
# fhe-math/src/ntt/native.rs


_ROOT_CACHE: Dict[tuple, int] = {}


def primitive_root(n: int, p: int) -> int:
    """native.rs:320-336 `primitive_root`: the first of 100 ChaCha8(seed 0)
    draws whose lambda-th power is a primitive 2n-th root of unity."""
    key = (n, p)
    if key in _ROOT_CACHE:
        return _ROOT_CACHE[key]
    lam = (p - 1) // (2 * n)
    rng = ChaChaRng.seed_from_u64(0)
    for _ in range(100):
        root = rng.random_range_u64(0, p)
        root = pow(root, lam, p) if lam > 1 else (root if lam == 1 else 1)
        # native.rs:341-348 `is_primitive_root`
        if pow(root, 2 * n, p) == 1 and pow(root, n, p) != 1:
            _ROOT_CACHE[key] = root
            return root
    raise RuntimeError("Couldn't find primitive root")


class NttOperator:
    """ntt/native.rs:15-73 `NttOperator` (tables) + forward/backward loops."""

    def __init__(self, p: Modulus, size: int, root: Optional[int] = None):
        if not supports_ntt(p.p, size):
            raise ValueError("NTT not supported")
        self.p = p
        self.size = size
        self.size_inv = p.inv(size)
        self.omega = primitive_root(size, p.p) if root is None else root
        omega_inv = p.inv(self.omega)
        self.omegas = np.empty(size, dtype=np.uint64)
        self.omegas_shoup = np.empty(size, dtype=np.uint64)
        self.zetas_inv = np.empty(size, dtype=np.uint64)
        self.zetas_inv_shoup = np.empty(size, dtype=np.uint64)
        lib().ora_ntt_tables(_p(p.fields), size, self.omega, omega_inv, _p(self.omegas), _p(self.omegas_shoup),
                             _p(self.zetas_inv), _p(self.zetas_inv_shoup))
        self.size_inv_shoup = p.shoup(self.size_inv)

    def forward(self, a: np.ndarray):
        """native.rs:77-102 (rows of a 2-D array are transformed independently)."""
        rows = a.size // self.size
        lib().ora_ntt_forward(_p(self.p.fields), self.size, _p(self.omegas), _p(self.omegas_shoup), _p(a), rows, 0)

    def forward_vt_lazy(self, a: np.ndarray):
        """native.rs:142-175: output in [0, 4p)."""
        rows = a.size // self.size
        lib().ora_ntt_forward(_p(self.p.fields), self.size, _p(self.omegas), _p(self.omegas_shoup), _p(a), rows, 1)

    def backward(self, a: np.ndarray):
        """native.rs:106-132."""
        rows = a.size // self.size
        lib().ora_ntt_backward(_p(self.p.fields), self.size, _p(self.zetas_inv), _p(self.zetas_inv_shoup),
                               self.size_inv, self.size_inv_shoup, _p(a), rows)


_OP_CACHE: Dict[tuple, NttOperator] = {}


def ntt_operator(p: int, n: int) -> NttOperator:
    key = (p, n)
    if key not in _OP_CACHE:
        _OP_CACHE[key] = NttOperator(Modulus(p), n)
    return _OP_CACHE[key]


# ---------------------------------------------------------------------------
# fhe-math/src/rns


class RnsContext:
    """rns/mod.rs:23-146 `RnsContext`."""

    def __init__(self, moduli: Sequence[int]):
        if len(moduli) == 0:
            raise ValueError("The list of moduli is empty")
        for i in range(len(moduli)):
            for j in range(len(moduli)):
                if i != j and math.gcd(moduli[i], moduli[j]) != 1:
                    raise ValueError("The moduli are not coprime")
        self.moduli_u64 = [int(m) for m in moduli]
        self.moduli = [Modulus(m) for m in self.moduli_u64]
        self.product = 1
        for m in self.moduli_u64:
            self.product *= m
        self.q_star = [self.product // m for m in self.moduli_u64]
        self.q_tilde = [pow(qs % m, -1, m) for qs, m in zip(self.q_star, self.moduli_u64)]
        self.garner = [qs * qt for qs, qt in zip(self.q_star, self.q_tilde)]

    def modulus(self) -> int:
        return self.product

    def project(self, a: int) -> List[int]:
        return [a % m for m in self.moduli_u64]

    def lift(self, rests: Sequence[int]) -> int:
        return sum(int(g) * int(r) for g, r in zip(self.garner, rests)) % self.product

    def get_garner(self, i: int) -> int:
        return self.garner[i]


@dataclass
class ScalingFactor:
    """rns/scaler.rs:19-47 `ScalingFactor`."""

    numerator: int
    denominator: int

    def __post_init__(self):
        assert self.denominator != 0
        self.is_one = self.numerator == self.denominator

    @staticmethod
    def one() -> "ScalingFactor":
        return ScalingFactor(1, 1)


def extract_projection_and_theta(ctx: RnsContext, inp: int, numerator: int, denominator: int, round_up: bool):
    """rns/scaler.rs:183-229 `extract_projection_and_theta`."""
    gamma = (numerator * inp + (denominator >> 1)) // denominator
    projected = ctx.project(gamma)
    theta = (numerator * inp) % denominator
    theta_sign = False
    if denominator > 1:
        if denominator & 1 == 1:
            if theta > (denominator >> 1):
                theta_sign = True
                theta = denominator - theta
        else:
            if theta >= (denominator >> 1):
                theta_sign = True
                theta = denominator - theta
    if round_up:
        if theta_sign:
            theta = (theta << 127) // denominator
        else:
            theta = ((theta << 127) + denominator - 1) // denominator
    elif theta_sign:
        theta = ((theta << 127) + denominator - 1) // denominator
    else:
        theta = (theta << 127) // denominator
    theta_hi = theta >> 64
    theta_lo = theta - (theta_hi << 64)
    return projected, theta_lo, theta_hi, theta_sign


class RnsScaler:
    """rns/scaler.rs:51-175 `RnsScaler::new`; `scale` runs in oracle.cpp."""

    def __init__(self, frm: RnsContext, to: RnsContext, factor: ScalingFactor):
        self.frm, self.to, self.factor = frm, to, factor
        n, d = factor.numerator, factor.denominator
        gamma, tg_lo, tg_hi, tg_sign = extract_projection_and_theta(to, frm.product, n, d, False)
        self.gamma = _u64(gamma)
        self.gamma_shoup = _u64([q.shoup(g) for q, g in zip(to.moduli, gamma)])
        self.theta_gamma = (tg_lo, tg_hi, tg_sign)
        omega = np.zeros((len(to.moduli), len(frm.moduli)), dtype=np.uint64)
        omega_shoup = np.zeros_like(omega)
        to_lo, to_hi, to_sign = [], [], []
        for i, g in enumerate(frm.garner):
            om_i, lo, hi, sg = extract_projection_and_theta(to, g, n, d, True)
            to_lo.append(lo)
            to_hi.append(hi)
            to_sign.append(int(sg))
            for j, qj in enumerate(to.moduli):
                v = om_i[j] % qj.p  # scaler.rs:123 (`reduce` of a value already < q_j)
                omega[j, i] = v
                omega_shoup[j, i] = qj.shoup(v)
        self.omega, self.omega_shoup = omega, omega_shoup
        self.theta_omega_lo, self.theta_omega_hi, self.theta_omega_sign = _u64(to_lo), _u64(to_hi), _u64(to_sign)
        # scaler.rs:130-142
        L = len(frm.moduli_u64)
        self.theta_garner_shift = min(
            min(191 - _next_pow2(q * L).bit_length() + 1 for q in frm.moduli_u64), 127)
        # scaler.rs:145-155
        lo, hi = [], []
        for g in frm.garner:
            theta = ((g << self.theta_garner_shift) + (frm.product >> 1)) // frm.product
            hi.append(theta >> 64)
            lo.append(theta & M64)
        self.theta_garner_lo, self.theta_garner_hi = _u64(lo), _u64(hi)
        self.to_moduli = _u64(np.concatenate([m.fields for m in to.moduli]))
        self._desc = OraScaler(
            len(frm.moduli), len(to.moduli), int(factor.is_one), _p(self.to_moduli), _p(self.gamma),
            _p(self.gamma_shoup), tg_lo, tg_hi, int(tg_sign), _p(self.omega), _p(self.omega_shoup),
            _p(self.theta_omega_lo), _p(self.theta_omega_hi), _p(self.theta_omega_sign),
            _p(self.theta_garner_lo), _p(self.theta_garner_hi), self.theta_garner_shift)

    def scale_columns(self, inp: np.ndarray, starting_index: int, out_len: int) -> np.ndarray:
        """rq/scaler.rs:84-93: `RnsScaler::scale` applied to every column of a
        [from_len][n] power-basis array."""
        assert inp.shape[0] == len(self.frm.moduli)
        n = inp.shape[1]
        out = np.zeros((out_len, n), dtype=np.uint64)
        inp = np.ascontiguousarray(inp)
        lib().ora_rns_scale(ctypes.byref(self._desc), _p(inp), _p(out), n, starting_index, out_len)
        return out

    def scale_new(self, rests: Sequence[int], size: int) -> List[int]:
        """rns/scaler.rs:237-241 `scale_new`."""
        r = _u64(rests)
        out = np.zeros(size, dtype=np.uint64)
        lib().ora_rns_scale_column(ctypes.byref(self._desc), _p(r), _p(out), 0, size)
        return [int(x) for x in out]


def _next_pow2(x: int) -> int:
    return 1 if x <= 1 else 1 << (x - 1).bit_length()


# ---------------------------------------------------------------------------
# fhe-math/src/rq


def bitrev(x: int, logn: int) -> int:
    return int(format(x, f"0{logn}b")[::-1], 2) if logn > 0 else 0


class Context:
    """rq/context.rs:9-156 `Context`."""

    def __init__(self, moduli: Sequence[int], degree: int):
        if degree < 8 or degree & (degree - 1):
            raise ValueError("The degree is not a power of two larger or equal to 8")
        self.moduli = [int(m) for m in moduli]
        self.degree = degree
        self.rns = RnsContext(self.moduli)
        self.q = self.rns.moduli
        self.ops = [ntt_operator(m, degree) for m in self.moduli]
        logn = degree.bit_length() - 1
        self.bitrev = np.array([bitrev(j, logn) for j in range(degree)], dtype=np.int64)
        q_last = self.moduli[-1]
        self.inv_last_qi_mod_qj = _u64([pow(q_last % qi.p, -1, qi.p) for qi in self.q[:-1]])
        self.inv_last_qi_mod_qj_shoup = _u64(
            [qi.shoup(int(v)) for qi, v in zip(self.q[:-1], self.inv_last_qi_mod_qj)])
        self._next = None

    @property
    def next_context(self) -> Optional["Context"]:
        if self._next is None and len(self.moduli) >= 2:
            self._next = Context(self.moduli[:-1], self.degree)
        return self._next

    def __eq__(self, other):
        return isinstance(other, Context) and other.moduli == self.moduli and other.degree == self.degree

    def __hash__(self):
        return hash((tuple(self.moduli), self.degree))

    def modulus(self) -> int:
        return self.rns.product

    def niterations_to(self, ctx: "Context") -> int:
        """rq/context.rs:120-141."""
        if ctx == self:
            return 0
        if ctx.degree == self.degree and len(ctx.moduli) < len(self.moduli) and \
                self.moduli[:len(ctx.moduli)] == ctx.moduli:
            return len(self.moduli) - len(ctx.moduli)
        raise ValueError("InvalidContext")


class SubstitutionExponent:
    """rq/mod.rs:87-121 `SubstitutionExponent`."""

    def __init__(self, ctx: Context, exponent: int):
        exponent = exponent % (2 * ctx.degree)
        if exponent & 1 == 0:
            raise ValueError("The exponent should be odd modulo 2 * degree")
        self.exponent = exponent
        self.ctx = ctx
        logn = ctx.degree.bit_length() - 1
        mask = ctx.degree - 1
        power = (exponent - 1) // 2
        pb = []
        for _ in range(ctx.degree):
            pb.append(bitrev(power & mask, logn))
            power += exponent
        self.power_bitrev = np.array(pb, dtype=np.int64)


POWER_BASIS, NTT, NTT_SHOUP = "PowerBasis", "Ntt", "NttShoup"


class Poly:
    """rq/mod.rs:124-132 `Poly<R>`: coefficients [L][N] (limb-major)."""

    def __init__(self, ctx: Context, coefficients: np.ndarray, representation: str):
        assert coefficients.shape == (len(ctx.moduli), ctx.degree)
        self.ctx = ctx
        self.coefficients = np.ascontiguousarray(coefficients, dtype=np.uint64)
        self.representation = representation
        self.coefficients_shoup = None
        if representation == NTT_SHOUP:
            self.compute_coefficients_shoup()

    def copy(self) -> "Poly":
        p = Poly(self.ctx, self.coefficients.copy(), self.representation)
        return p

    @staticmethod
    def zero(ctx: Context, representation: str) -> "Poly":
        return Poly(ctx, np.zeros((len(ctx.moduli), ctx.degree), dtype=np.uint64), representation)

    def compute_coefficients_shoup(self):
        """rq/mod.rs:209-223."""
        self.coefficients_shoup = np.stack([qi.shoup_vec(self.coefficients[i]) for i, qi in enumerate(self.ctx.q)])

    @staticmethod
    def random(ctx: Context, representation: str, rng: np.random.Generator) -> "Poly":
        """rq/mod.rs:226-237 (numpy stream in place of the caller's RNG)."""
        c = np.stack([rng.integers(0, m, ctx.degree, dtype=np.uint64) for m in ctx.moduli])
        return Poly(ctx, c, representation)

    @staticmethod
    def random_from_seed(ctx: Context, seed: bytes, representation: str = NTT) -> "Poly":
        """rq/mod.rs:239-257."""
        p = Poly(ctx, random_from_seed(ctx, seed), representation)
        if representation == NTT_SHOUP:
            p.compute_coefficients_shoup()
        return p

    @staticmethod
    def small(ctx: Context, representation: str, variance: int, rng: np.random.Generator) -> "Poly":
        """rq/mod.rs:263-285: CBD coefficients, then the representation."""
        coeffs = sample_vec_cbd(ctx.degree, variance, rng)
        p = Poly.from_i64(ctx, coeffs)
        if representation == NTT:
            p.into_ntt()
        elif representation == NTT_SHOUP:
            p.into_ntt()
            p.representation = NTT_SHOUP
            p.compute_coefficients_shoup()
        return p

    @staticmethod
    def from_i64(ctx: Context, values: np.ndarray) -> "Poly":
        """rq/convert.rs:296-318 `TryConvertFrom<&[i64]>` (power basis)."""
        v = np.asarray(values, dtype=np.int64)
        c = np.zeros((len(ctx.moduli), ctx.degree), dtype=np.uint64)
        for i, m in enumerate(ctx.moduli):
            c[i, :len(v)] = np.mod(v.astype(object), m).astype(np.uint64)
        return Poly(ctx, c, POWER_BASIS)

    @staticmethod
    def from_u64(ctx: Context, values: np.ndarray) -> "Poly":
        """rq/convert.rs:137-177 `TryConvertFrom<Vec<u64>>` with at most `degree` values."""
        v = np.asarray(values, dtype=np.uint64)
        c = np.zeros((len(ctx.moduli), ctx.degree), dtype=np.uint64)
        for i, qi in enumerate(ctx.q):
            row = np.zeros(ctx.degree, dtype=np.uint64)
            row[:len(v)] = v
            qi.reduce_vec(row)
            c[i] = row
        return Poly(ctx, c, POWER_BASIS)

    @staticmethod
    def from_biguints(ctx: Context, values: Sequence[int]) -> "Poly":
        """rq/convert.rs:326-364 (`&[BigUint]`)."""
        c = np.zeros((len(ctx.moduli), ctx.degree), dtype=np.uint64)
        for j, x in enumerate(values):
            for i, m in enumerate(ctx.moduli):
                c[i, j] = int(x) % m
        return Poly(ctx, c, POWER_BASIS)

    def to_biguints(self) -> List[int]:
        """rq/convert.rs:477-499: CRT lift of every column."""
        cols = self.coefficients.T.tolist()
        return [self.ctx.rns.lift(col) for col in cols]

    # representation changes (rq/mod.rs:294-313, 488-579)
    def into_ntt(self) -> "Poly":
        assert self.representation == POWER_BASIS
        for i, op in enumerate(self.ctx.ops):
            row = self.coefficients[i]
            op.forward(row)
        self.representation = NTT
        return self

    def into_power_basis(self) -> "Poly":
        assert self.representation in (NTT, NTT_SHOUP)
        for i, op in enumerate(self.ctx.ops):
            op.backward(self.coefficients[i])
        self.representation = POWER_BASIS
        self.coefficients_shoup = None
        return self

    def into_ntt_shoup(self) -> "Poly":
        if self.representation == POWER_BASIS:
            self.into_ntt()
        self.representation = NTT_SHOUP
        self.compute_coefficients_shoup()
        return self

    # arithmetic (rq/ops.rs)
    def __iadd__(self, other: "Poly"):
        assert self.ctx == other.ctx
        for i, qi in enumerate(self.ctx.q):
            qi.add_vec(self.coefficients[i], other.coefficients[i])
        return self

    def __isub__(self, other: "Poly"):
        assert self.ctx == other.ctx
        for i, qi in enumerate(self.ctx.q):
            qi.sub_vec(self.coefficients[i], other.coefficients[i])
        return self

    def __add__(self, other: "Poly") -> "Poly":
        r = self.copy()
        r += other
        return r

    def __sub__(self, other: "Poly") -> "Poly":
        r = self.copy()
        r -= other
        return r

    def __neg__(self) -> "Poly":
        r = self.copy()
        for i, qi in enumerate(self.ctx.q):
            qi.neg_vec(r.coefficients[i])
        return r

    def mul_assign(self, other: "Poly"):
        """rq/ops.rs:174-245: Ntt x Ntt (Barrett/opt) or Ntt x NttShoup (Shoup)."""
        assert self.ctx == other.ctx and self.representation == NTT
        if other.representation == NTT_SHOUP:
            for i, qi in enumerate(self.ctx.q):
                qi.mul_shoup_vec(self.coefficients[i], other.coefficients[i], other.coefficients_shoup[i])
        else:
            assert other.representation == NTT
            for i, qi in enumerate(self.ctx.q):
                qi.mul_vec(self.coefficients[i], other.coefficients[i])
        return self

    def __mul__(self, other):
        r = self.copy()
        if isinstance(other, Poly):
            r.mul_assign(other)
        else:
            r.scalar_mul_assign(int(other))
        return r

    def scalar_mul_assign(self, big: int):
        """rq/ops.rs:297-352 `MulAssign<&BigUint>` (CRT projection, Shoup)."""
        for i, qi in enumerate(self.ctx.q):
            qi.scalar_mul_vec(self.coefficients[i], big % qi.p)
        return self

    def substitute(self, e: SubstitutionExponent) -> "Poly":
        """rq/mod.rs:319-369 `substitute`."""
        q = Poly.zero(self.ctx, self.representation)
        if self.representation in (NTT, NTT_SHOUP):
            q.coefficients[:, self.ctx.bitrev] = self.coefficients[:, e.power_bitrev]
            if self.representation == NTT_SHOUP:
                q.compute_coefficients_shoup()
        else:
            n = self.ctx.degree
            mask = n - 1
            idx = (np.arange(n, dtype=object) * e.exponent)
            dest = np.array([int(x) & mask for x in idx], dtype=np.int64)
            neg = np.array([(int(x) & n) != 0 for x in idx])
            for i, qi in enumerate(self.ctx.q):
                row = np.zeros(n, dtype=np.uint64)
                src = self.coefficients[i]
                pos_vals = src.copy()
                neg_vals = src.copy()
                qi.neg_vec(neg_vals)
                vals = np.where(neg, neg_vals, pos_vals)
                row[dest] = vals  # x -> x^e is a bijection on indices mod n
                q.coefficients[i] = row
        return q

    def switch_down(self) -> "Poly":
        """rq/mod.rs:390-448 `switch_down` (power basis)."""
        assert self.representation == POWER_BASIS
        nxt = self.ctx.next_context
        if nxt is None:
            raise ValueError("NoMoreContext")
        L, n = len(self.ctx.moduli), self.ctx.degree
        mods = _u64(np.concatenate([q.fields for q in self.ctx.q]))
        out = np.zeros((L - 1, n), dtype=np.uint64)
        lib().ora_switch_down(_p(mods), L, n, _p(self.ctx.inv_last_qi_mod_qj),
                              _p(self.ctx.inv_last_qi_mod_qj_shoup), _p(self.coefficients), _p(out))
        self.coefficients = out
        self.ctx = nxt
        return self

    def switch_down_to(self, ctx: Context) -> "Poly":
        """rq/mod.rs:455-462."""
        for _ in range(self.ctx.niterations_to(ctx)):
            self.switch_down()
        assert self.ctx == ctx
        return self

    def scale(self, scaler: "Scaler") -> "Poly":
        return scaler.scale(self)


class Scaler:
    """rq/scaler.rs:17-126 `Scaler`."""

    def __init__(self, frm: Context, to: Context, factor: ScalingFactor):
        if frm.degree != to.degree:
            raise ValueError("Incompatible degrees")
        self.frm, self.to = frm, to
        if factor.is_one:
            ncm = 0
            for a, b in zip(frm.moduli, to.moduli):
                if a != b:
                    break
                ncm += 1
            self.number_common_moduli = ncm
        else:
            self.number_common_moduli = 0
        self.scaler = RnsScaler(frm.rns, to.rns, factor)

    def scale(self, p: Poly) -> Poly:
        if p.ctx != self.frm:
            raise ValueError("The input polynomial does not have the correct context")
        ncm = self.number_common_moduli
        out = np.zeros((len(self.to.moduli), self.to.degree), dtype=np.uint64)
        if ncm > 0:
            out[:ncm] = p.coefficients[:ncm]
        if ncm < len(self.to.moduli):
            needs_transform = p.representation != POWER_BASIS
            src = p.coefficients.copy()
            if needs_transform:
                for i, op in enumerate(p.ctx.ops):
                    op.backward(src[i])
            new = self.scaler.scale_columns(src, ncm, len(self.to.moduli) - ncm)
            if needs_transform:
                for k, op in enumerate(self.to.ops[ncm:]):
                    op.forward(new[k])
            out[ncm:] = new
        rep = POWER_BASIS if p.representation == POWER_BASIS else NTT
        return Poly(self.to, out, rep)


class Switcher:
    """rq/switcher.rs:11-26 `Switcher`."""

    def __init__(self, frm: Context, to: Context):
        self.scaler = Scaler(frm, to, ScalingFactor(to.modulus(), frm.modulus()))

    def switch(self, p: Poly) -> Poly:
        return self.scaler.scale(p)


# ---------------------------------------------------------------------------
# fhe-util sampling


def sample_vec_cbd(size: int, variance: int, rng: np.random.Generator) -> np.ndarray:
    """fhe-util/src/lib.rs:22-55 `sample_vec_cbd` over a numpy u64 stream.

    The reference keeps a bit pool fed by 64-bit draws (appended above the
    bits already pooled) and consumes 4*variance bits per sample: the first
    2*variance are added, the next 2*variance subtracted. That is the same as
    cutting the concatenated little-endian bit stream of the draws into
    consecutive 4*variance-bit chunks, which is what this does."""
    if not (1 <= variance <= 16):
        raise ValueError("The variance should be between 1 and 16")
    nb = 4 * variance
    ndraws = (size * nb + 63) // 64 + 2
    draws = rng.integers(0, 1 << 64, size=ndraws, dtype=np.uint64, endpoint=False)
    return _cbd_from_draws(draws, size, variance)


def _cbd_from_draws(draws: np.ndarray, size: int, variance: int) -> np.ndarray:
    nb = 4 * variance
    bits = np.unpackbits(np.ascontiguousarray(draws, dtype=np.uint64).view(np.uint8),
                         bitorder="little")[: size * nb].reshape(size, nb)
    half = 2 * variance
    return bits[:, :half].sum(axis=1).astype(np.int64) - bits[:, half:].sum(axis=1).astype(np.int64)


def sample_vec_cbd_from_seed(size: int, variance: int, seed: bytes) -> np.ndarray:
    """`sample_vec_cbd` (fhe-util/src/lib.rs:22-55) driven by the next_u64
    stream of ChaCha8Rng::from_seed(seed) (rand_chacha 0.9.0): it takes
    ceil(4 * variance * size / 64) draws."""
    if not (1 <= variance <= 16):
        raise ValueError("The variance should be between 1 and 16")
    key = [int.from_bytes(seed[4 * i:4 * i + 4], "little") for i in range(8)]
    ndraws = (size * 4 * variance + 63) // 64
    return _cbd_from_draws(chacha_u64_draws(key, 0, ndraws), size, variance)


# ---------------------------------------------------------------------------
# fhe/src/bfv


class CipherPlainContext:
    """fhe/src/bfv/context/cipher_plain_context.rs:9-28 (built by parameters.rs:509-562)."""

    def __init__(self, par: "BfvParameters", level_moduli: List[int], cipher_ctx: Context):
        t = par.plaintext
        delta_rests = []
        for m in level_moduli:
            neg_t = (-(t % m)) % m
            delta_rests.append(pow(neg_t, -1, m))
        rns = RnsContext(level_moduli)
        self.delta = Poly.from_biguints(cipher_ctx, [rns.lift(delta_rests)]).into_ntt_shoup()
        self.q_mod_t = rns.modulus() % t
        self.plain_threshold = (t + 1) >> 1
        self.scaler = Scaler(cipher_ctx, par.plaintext_context, ScalingFactor(t, rns.modulus()))
        self.ciphertext_context = cipher_ctx


class MultiplicationParameters:
    """parameters.rs:694-717."""

    def __init__(self, frm: Context, to: Context, up: ScalingFactor, down: ScalingFactor):
        self.extender = Scaler(frm, to, up)
        self.down_scaler = Scaler(to, frm, down)
        self.frm, self.to = frm, to


class BfvParameters:
    """parameters.rs:76-641 `BfvParameters` built by `BfvParametersBuilder::build`."""

    def __init__(self, degree: int, plaintext: int, moduli: Optional[Sequence[int]] = None,
                 moduli_sizes: Optional[Sequence[int]] = None, variance: int = 10):
        if degree < 8 or degree & (degree - 1):
            raise ValueError("invalid degree")
        self.degree = degree
        self.plaintext = plaintext
        self.variance = variance
        if moduli is None:
            moduli = self.generate_moduli(list(moduli_sizes), degree)
        self.moduli = [int(m) for m in moduli]
        self.moduli_sizes = [m.bit_length() for m in self.moduli]
        t_bits = plaintext.bit_length()
        acc, count = 0, 0
        for size in self.moduli_sizes:  # parameters.rs:480-491
            acc += size
            count += 1
            if acc >= t_bits + 60:
                break
        count = min(max(count, 1), len(self.moduli))
        self.plaintext_context = Context(self.moduli[:count], degree)
        self.ntt_operator = ntt_operator(plaintext, degree) if supports_ntt(plaintext, degree) else None
        L = len(self.moduli)
        self.contexts = [Context(self.moduli[:L - i], degree) for i in range(L)]
        self._cp = {}
        # parameters.rs:585-593: n+1 62-bit moduli for multiplication.
        ext, ub = [], 1 << 62
        while len(ext) != L + 1:
            ub = generate_prime(62, 2 * degree, ub)
            if ub not in ext and ub not in self.moduli:
                ext.append(ub)
        self.extended_basis = ext
        self._mp = {}
        # parameters.rs:616-629: SIMD index map.
        row_size = degree >> 1
        m = degree << 1
        pos = 1
        logn = degree.bit_length() - 1
        self.matrix_reps_index_map = np.zeros(degree, dtype=np.int64)
        for i in range(row_size):
            index1 = (pos - 1) >> 1
            index2 = (m - pos - 1) >> 1
            self.matrix_reps_index_map[i] = bitrev(index1, logn)
            self.matrix_reps_index_map[row_size | i] = bitrev(index2, logn)
            pos = (pos * 3) & (m - 1)

    @staticmethod
    def generate_moduli(sizes: List[int], degree: int) -> List[int]:
        """parameters.rs:383-423."""
        moduli = []
        for size in sizes:
            ub = 1 << size
            while True:
                prime = generate_prime(size, 2 * degree, ub)
                if prime is None:
                    raise ValueError("NotEnoughPrimes")
                if prime not in moduli:
                    moduli.append(prime)
                    break
                ub = prime
        return moduli

    def max_level(self) -> int:
        return len(self.moduli) - 1

    def context_at_level(self, level: int) -> Context:
        if level > self.max_level():
            raise ValueError("InvalidLevel")
        return self.contexts[level]

    def level_of_context(self, ctx: Context) -> int:
        return self.contexts[0].niterations_to(ctx)

    def cipher_plain_context(self, level: int) -> CipherPlainContext:
        if level not in self._cp:
            ctx = self.contexts[level]
            self._cp[level] = CipherPlainContext(self, ctx.moduli, ctx)
        return self._cp[level]

    def mul_params(self, level: int) -> MultiplicationParameters:
        """parameters.rs:596-612."""
        if level not in self._mp:
            sizes = self.moduli_sizes[:len(self.moduli) - level]
            n_moduli = (sum(sizes) + 60 + 61) // 62
            mul_moduli = self.moduli[:len(self.moduli) - level] + self.extended_basis[:n_moduli]
            mul_ctx = Context(mul_moduli, self.degree)
            ctx = self.contexts[level]
            self._mp[level] = MultiplicationParameters(ctx, mul_ctx, ScalingFactor.one(),
                                                       ScalingFactor(self.plaintext, ctx.modulus()))
        return self._mp[level]


class Plaintext:
    """plaintext.rs:36-98 (Small plaintext modulus only)."""

    def __init__(self, par: BfvParameters, value: np.ndarray, level: int, encoding: Optional[str]):
        self.par, self.value, self.level, self.encoding = par, _u64(value), level, encoding

    @staticmethod
    def encode(values: Sequence[int], encoding: str, par: BfvParameters, level: int = 0) -> "Plaintext":
        """plaintext_vec.rs:40-100 (`simd` or `poly`)."""
        n = par.degree
        v = np.zeros(n, dtype=np.uint64)
        vals = _u64(values)
        if encoding == "poly":
            v[:len(vals)] = vals
        else:
            v[par.matrix_reps_index_map[:len(vals)]] = vals
            par.ntt_operator.backward(v)
        return Plaintext(par, v, level, encoding)

    def decode(self, encoding: Optional[str] = None) -> np.ndarray:
        """plaintext.rs FheDecoder<Plaintext> for Vec<u64>."""
        enc = encoding or self.encoding
        w = self.value.copy()
        if enc == "poly":
            return w
        self.par.ntt_operator.forward(w)
        return w[self.par.matrix_reps_index_map]

    def to_poly(self) -> Poly:
        """plaintext.rs:71-98."""
        cp = self.par.cipher_plain_context(self.level)
        ctx = self.par.context_at_level(self.level)
        m_v = self.value.copy()
        Modulus(self.par.plaintext).scalar_mul_vec(m_v, cp.q_mod_t)
        m = Poly.from_u64(ctx, m_v).into_ntt()
        m.mul_assign(cp.delta)
        return m


class Ciphertext:
    """ciphertext.rs:17-119 `Ciphertext`."""

    def __init__(self, par: BfvParameters, c: List[Poly], level: int):
        self.par, self.c, self.level = par, c, level

    def __len__(self):
        return len(self.c)

    def __getitem__(self, i):
        return self.c[i]

    def copy(self) -> "Ciphertext":
        return Ciphertext(self.par, [p.copy() for p in self.c], self.level)

    def to_array(self) -> np.ndarray:
        return np.stack([p.coefficients for p in self.c])

    @staticmethod
    def from_array(par: BfvParameters, arr: np.ndarray, level: int) -> "Ciphertext":
        ctx = par.context_at_level(level)
        return Ciphertext(par, [Poly(ctx, arr[i], NTT) for i in range(arr.shape[0])], level)

    def switch_down(self) -> "Ciphertext":
        """ciphertext.rs:86-97."""
        if self.level < self.par.max_level():
            for i, ci in enumerate(self.c):
                pb = ci.copy().into_power_basis()
                pb.switch_down()
                self.c[i] = pb.into_ntt()
            self.level += 1
        return self

    def __add__(self, other: "Ciphertext") -> "Ciphertext":
        """ops/mod.rs:15-43."""
        assert self.level == other.level and len(self) == len(other)
        return Ciphertext(self.par, [a + b for a, b in zip(self.c, other.c)], self.level)

    def __mul__(self, other: "Ciphertext") -> "Ciphertext":
        """ops/mod.rs:259-342 (`&ct * &ct` without relinearization)."""
        mp = self.par.mul_params(self.level)
        c00 = self[0].scale(mp.extender)
        c01 = self[1].scale(mp.extender)
        c10 = other[0].scale(mp.extender)
        c11 = other[1].scale(mp.extender)
        c0 = c00 * c10
        c1 = c00 * c11
        c1 += c01 * c10
        c2 = c01 * c11
        return Ciphertext(self.par, [c.scale(mp.down_scaler) for c in (c0, c1, c2)], self.level)


class SecretKey:
    """keys/secret_key.rs:24-270 `SecretKey`."""

    def __init__(self, par: BfvParameters, coeffs: np.ndarray):
        self.par = par
        self.coeffs = np.asarray(coeffs, dtype=np.int64)

    @staticmethod
    def random(par: BfvParameters, rng: np.random.Generator) -> "SecretKey":
        """secret_key.rs:44-47 (CBD with the parameters' variance)."""
        return SecretKey(par, sample_vec_cbd(par.degree, par.variance, rng))

    @staticmethod
    def ternary(par: BfvParameters, rng: np.random.Generator) -> "SecretKey":
        """A secret uniform in {-1, 0, 1} (the benchmark's ternary secret)."""
        return SecretKey(par, rng.integers(-1, 2, par.degree).astype(np.int64))

    def s_ntt(self, ctx: Context) -> Poly:
        return Poly.from_i64(ctx, self.coeffs).into_ntt()

    def encrypt_poly(self, m: Poly, rng: np.random.Generator) -> Ciphertext:
        """secret_key.rs:102-138."""
        level = self.par.level_of_context(m.ctx)
        s = self.s_ntt(m.ctx)
        a = Poly.random(m.ctx, NTT, rng)
        a_s = a * s
        b = Poly.small(m.ctx, NTT, self.par.variance, rng)
        b -= a_s
        b += m
        return Ciphertext(self.par, [b, a], level)

    def encrypt(self, pt: Plaintext, rng: np.random.Generator) -> Ciphertext:
        return self.encrypt_poly(pt.to_poly(), rng)

    def encrypt_with(self, pt: Plaintext, a_ntt: np.ndarray, e: np.ndarray) -> Ciphertext:
        """secret_key.rs:102-138 with the randomness given: a (uniform, Ntt)
        and the small error coefficients e; b = e - a s + m."""
        m = pt.to_poly()
        s = self.s_ntt(m.ctx)
        a = Poly(m.ctx, np.array(a_ntt, dtype=np.uint64), NTT)
        b = Poly.from_i64(m.ctx, np.asarray(e, dtype=np.int64)).into_ntt()
        b -= a * s
        b += m
        return Ciphertext(self.par, [b, a], self.par.level_of_context(m.ctx))

    def decrypt(self, ct: Ciphertext) -> Plaintext:
        """secret_key.rs:200-280."""
        ctx = ct[0].ctx
        s = self.s_ntt(ctx)
        si = s.copy()
        c = ct[0].copy()
        for i in range(1, len(ct)):
            cis = ct[i] * si
            c += cis
            if i + 1 < len(ct):
                si.mul_assign(s)
        c.into_power_basis()
        d = c.scale(self.par.cipher_plain_context(ct.level).scaler)
        t = self.par.plaintext
        v = d.coefficients.reshape(-1).astype(object) + t
        w = v[:self.par.degree]
        w = np.array([int(x) % self.par.moduli[0] % t for x in w], dtype=np.uint64)
        return Plaintext(self.par, w, ct.level, None)

    def measure_noise(self, ct: Ciphertext) -> int:
        """secret_key.rs:63-100."""
        pt = self.decrypt(ct)
        pt.level = ct.level
        m = pt.to_poly()
        s = self.s_ntt(ct[0].ctx)
        si = s.copy()
        c = ct[0].copy()
        for i in range(1, len(ct)):
            c += ct[i] * si
            si.mul_assign(s)
        c -= m
        c.into_power_basis()
        q = ct[0].ctx.modulus()
        return max(min(x.bit_length(), (q - x).bit_length()) for x in c.to_biguints())


def decomposition_log_base(ctx: Context) -> int:
    """key_switching_key.rs:70-73: half the bit length of the (single) key
    modulus rounded up to a power of two."""
    log_modulus = _next_pow2(ctx.moduli[0]).bit_length() - 1
    return log_modulus // 2


def decomposition_digits(p: Poly, log_base: int) -> np.ndarray:
    """key_switching_key.rs:300-314: the base-2^log_base digits of the
    coefficients (every limb's row in turn), one row per digit."""
    log_modulus = _next_pow2(p.ctx.moduli[0]).bit_length() - 1
    coeffs = p.coefficients.reshape(-1).copy()
    mask = np.uint64((1 << log_base) - 1)
    out = []
    for _ in range(-(-log_modulus // log_base)):
        out.append(coeffs & mask)
        coeffs >>= np.uint64(log_base)
    return np.stack(out)


class KeySwitchingKey:
    """keys/key_switching_key.rs:21-329: RNS digits (one per ciphertext
    modulus), or for a single-modulus key context the bit decomposition with
    base 2^log_base (generate_c0_decomposition, key_switch_decomposition)."""

    def __init__(self, sk: SecretKey, frm: Poly, ciphertext_level: int, ksk_level: int,
                 rng: np.random.Generator, seed: Optional[bytes] = None):
        par = sk.par
        self.par = par
        self.ctx_ksk = par.context_at_level(ksk_level)
        self.ctx_ciphertext = par.context_at_level(ciphertext_level)
        self.ciphertext_level, self.ksk_level = ciphertext_level, ksk_level
        if frm.ctx != self.ctx_ksk:
            raise ValueError("Incorrect context for polynomial from")
        self.log_base = 0
        size = len(self.ctx_ciphertext.moduli)
        if len(self.ctx_ksk.moduli) == 1:
            # key_switching_key.rs:70-76
            self.log_base = decomposition_log_base(self.ctx_ksk)
            log_modulus = _next_pow2(self.ctx_ksk.moduli[0]).bit_length() - 1
            size = -(-log_modulus // self.log_base)
        # generate_c1 (108-123): uniform NttShoup polys, from the key's seed
        # when one is given (as the reference always does), else drawn from
        # the numpy generator.
        self.seed = None if seed is None else bytes(seed)
        if seed is None:
            self.c1 = [Poly.random(self.ctx_ksk, NTT_SHOUP, rng) for _ in range(size)]
        else:
            self.c1 = [Poly.random_from_seed(self.ctx_ksk, s, NTT_SHOUP) for s in ksk_c1_seeds(seed, size)]
        # generate_c0 (126-169) / generate_c0_decomposition (172-211): the
        # i-th c0 carries `from` times the i-th Garner coefficient, or times
        # 2^(i * log_base).
        s = sk.s_ntt(self.ctx_ksk)
        rns = None if self.log_base else RnsContext(par.moduli[:size])
        self.c0 = []
        for i, c1i in enumerate(self.c1):
            a_s = Poly(self.ctx_ksk, c1i.coefficients.copy(), NTT)
            a_s.mul_assign(s)
            a_s.into_power_basis()
            b = Poly.small(self.ctx_ksk, POWER_BASIS, par.variance, rng)
            b -= a_s
            b += frm * (1 << (i * self.log_base) if self.log_base else rns.get_garner(i))
            self.c0.append(b.into_ntt_shoup())

    @staticmethod
    def from_arrays(par: BfvParameters, c0: np.ndarray, c1: np.ndarray, ciphertext_level: int,
                    ksk_level: int, log_base: int = 0) -> "KeySwitchingKey":
        k = KeySwitchingKey.__new__(KeySwitchingKey)
        k.par = par
        k.ctx_ksk = par.context_at_level(ksk_level)
        k.ctx_ciphertext = par.context_at_level(ciphertext_level)
        k.ciphertext_level, k.ksk_level = ciphertext_level, ksk_level
        k.log_base = log_base
        k.c0 = [Poly(k.ctx_ksk, c0[i], NTT_SHOUP) for i in range(c0.shape[0])]
        k.c1 = [Poly(k.ctx_ksk, c1[i], NTT_SHOUP) for i in range(c1.shape[0])]
        return k

    def c0_array(self) -> np.ndarray:
        return np.stack([p.coefficients for p in self.c0])

    def c1_array(self) -> np.ndarray:
        return np.stack([p.coefficients for p in self.c1])

    def key_switch(self, p: Poly):
        """key_switching_key.rs:214-241 (loop in oracle.cpp); for
        decomposition keys key_switching_key.rs:292-329, the same loop over
        the base-2^log_base digits of the coefficients."""
        if p.ctx != self.ctx_ciphertext:
            raise ValueError("The input polynomial does not have the correct context.")
        rows = decomposition_digits(p, self.log_base) if self.log_base else p.coefficients
        rows = np.ascontiguousarray(rows, dtype=np.uint64)
        ctx = self.ctx_ksk
        n, Lk = ctx.degree, len(ctx.moduli)
        limbs = (OraKskLimb * Lk)()
        for j, (qj, op) in enumerate(zip(ctx.q, ctx.ops)):
            for f in range(5):
                limbs[j].mod[f] = int(qj.fields[f])
            limbs[j].omegas = _p(op.omegas)
            limbs[j].omegas_shoup = _p(op.omegas_shoup)
        c0 = np.ascontiguousarray(np.stack([k.coefficients for k in self.c0]))
        c0s = np.ascontiguousarray(np.stack([k.coefficients_shoup for k in self.c0]))
        c1 = np.ascontiguousarray(np.stack([k.coefficients for k in self.c1]))
        c1s = np.ascontiguousarray(np.stack([k.coefficients_shoup for k in self.c1]))
        out0 = np.zeros((Lk, n), dtype=np.uint64)
        out1 = np.zeros((Lk, n), dtype=np.uint64)
        lib().ora_key_switch(limbs, Lk, n, _p(rows), rows.shape[0], _p(c0), _p(c0s), _p(c1),
                             _p(c1s), _p(out0), _p(out1))
        return Poly(ctx, out0, NTT), Poly(ctx, out1, NTT)


class RelinearizationKey:
    """keys/relinearization_key.rs:22-106."""

    def __init__(self, sk: SecretKey, rng: np.random.Generator, ciphertext_level: int = 0, key_level: int = 0,
                 seed: Optional[bytes] = None):
        par = sk.par
        ctx_rk = par.context_at_level(key_level)
        ctx_ct = par.context_at_level(ciphertext_level)
        if len(ctx_rk.moduli) == 1:
            raise ValueError("These parameters do not support key switching")
        s = sk.s_ntt(ctx_ct)
        s2 = (s * s).into_power_basis()
        s2_up = Switcher(ctx_ct, ctx_rk).switch(s2)
        self.ksk = KeySwitchingKey(sk, s2_up, ciphertext_level, key_level, rng, seed)

    @staticmethod
    def from_ksk(ksk: KeySwitchingKey) -> "RelinearizationKey":
        rk = RelinearizationKey.__new__(RelinearizationKey)
        rk.ksk = ksk
        return rk

    def relinearizes_poly(self, c2: Poly):
        return self.ksk.key_switch(c2)

    def relinearizes(self, ct: Ciphertext) -> Ciphertext:
        """relinearization_key.rs:71-98."""
        if len(ct) != 3:
            raise ValueError("Only supports relinearization of ciphertext with 3 parts")
        if ct.level != self.ksk.ciphertext_level:
            raise ValueError("Ciphertext has incorrect level")
        c2 = ct[2].copy().into_power_basis()
        c0, c1 = self.relinearizes_poly(c2)
        if c0.ctx != ct[0].ctx:
            c0 = c0.into_power_basis().switch_down_to(ct[0].ctx).into_ntt()
            c1 = c1.into_power_basis().switch_down_to(ct[1].ctx).into_ntt()
        out = ct.copy()
        out.c[0] += c0
        out.c[1] += c1
        out.c = out.c[:2]
        return out


class GaloisKey:
    """keys/galois_key.rs:18-124."""

    def __init__(self, sk: SecretKey, exponent: int, ciphertext_level: int, galois_key_level: int,
                 rng: np.random.Generator, seed: Optional[bytes] = None):
        par = sk.par
        ctx_gk = par.context_at_level(galois_key_level)
        ctx_ct = par.context_at_level(ciphertext_level)
        self.element = SubstitutionExponent(ctx_ct, exponent)
        s = Poly.from_i64(ctx_ct, sk.coeffs)
        s_sub = s.substitute(self.element)
        s_sub_up = Switcher(ctx_ct, ctx_gk).switch(s_sub)
        self.ksk = KeySwitchingKey(sk, s_sub_up, ciphertext_level, galois_key_level, rng, seed)

    @staticmethod
    def from_ksk(exponent: int, ksk: KeySwitchingKey) -> "GaloisKey":
        gk = GaloisKey.__new__(GaloisKey)
        gk.element = SubstitutionExponent(ksk.ctx_ciphertext, exponent)
        gk.ksk = ksk
        return gk

    def relinearize(self, ct: Ciphertext) -> Ciphertext:
        """galois_key.rs:90-124 `relinearize_into` (same output as `relinearize`)."""
        assert len(ct) == 2
        c2 = ct[1].substitute(self.element).into_power_basis()
        out0, out1 = self.ksk.key_switch(c2)
        if out0.ctx != ct[0].ctx:
            out0 = out0.into_power_basis().switch_down_to(ct[0].ctx).into_ntt()
            out1 = out1.into_power_basis().switch_down_to(ct[1].ctx).into_ntt()
        out0 += ct[0].substitute(self.element)
        return Ciphertext(ct.par, [out0, out1], self.ksk.ciphertext_level)


class RGSWCiphertext:
    """bfv/rgsw_ciphertext.rs:19-160: the key-switching keys of m and of m s,
    m the plaintext's Ntt polynomial (`poly_ntt`, plaintext_vec.rs:76) in the
    power basis, both at the plaintext's level."""

    def __init__(self, sk: SecretKey, pt: Plaintext, rng: np.random.Generator):
        # rgsw_ciphertext.rs:101-121 (SecretKey::try_encrypt).
        level = pt.level
        ctx = sk.par.context_at_level(level)
        m_ntt = Poly.from_u64(ctx, pt.value).into_ntt()
        m = m_ntt.copy().into_power_basis()
        m_s = Poly.from_i64(ctx, sk.coeffs).into_ntt()
        m_s.mul_assign(m_ntt)
        m_s.into_power_basis()
        self.par, self.level = sk.par, level
        self.ksk0 = KeySwitchingKey(sk, m, level, level, rng)
        self.ksk1 = KeySwitchingKey(sk, m_s, level, level, rng)

    def external_product(self, ct: Ciphertext) -> Ciphertext:
        """rgsw_ciphertext.rs:123-153 (`&ct * &rgsw`)."""
        assert ct.level == self.level, "Ciphertext and RGSWCiphertext must have the same level"
        assert len(ct) == 2, "Ciphertext must have two parts"
        ct0 = ct[0].copy().into_power_basis()
        ct1 = ct[1].copy().into_power_basis()
        c0, c1 = self.ksk0.key_switch(ct0)
        c0p, c1p = self.ksk1.key_switch(ct1)
        return Ciphertext(self.par, [c0 + c0p, c1 + c1p], self.level)


def rotation_exponent(par: BfvParameters, i: int) -> int:
    """evaluation_key.rs:195-204: column rotation by i uses exponent 3^i mod 2N."""
    return pow(3, i, 2 * par.degree)


class EvaluationKey:
    """evaluation_key.rs:23-131 (row and column rotations)."""

    def __init__(self, sk: SecretKey, rng: np.random.Generator, columns: Sequence[int] = (),
                 row_rotation: bool = False, ciphertext_level: int = 0, evaluation_key_level: int = 0):
        par = sk.par
        self.par = par
        self.ciphertext_level, self.evaluation_key_level = ciphertext_level, evaluation_key_level
        self.rot_to_gk_exponent = {i: rotation_exponent(par, i) for i in columns}
        indices = set(self.rot_to_gk_exponent.values())
        if row_rotation:
            indices.add(2 * par.degree - 1)
        self.gk = {e: GaloisKey(sk, e, ciphertext_level, evaluation_key_level, rng) for e in sorted(indices)}

    def rotates_rows(self, ct: Ciphertext) -> Ciphertext:
        return self.gk[2 * self.par.degree - 1].relinearize(ct)

    @staticmethod
    def inner_sum_exponents(par: BfvParameters) -> List[int]:
        """evaluation_key.rs:56-83: the column rotations by 1, 2, 4, ... < N/2,
        then the row rotation, in the order computes_inner_sum applies them."""
        out, i = [], 1
        while i < par.degree // 2:
            out.append(rotation_exponent(par, i))
            i *= 2
        return out + [2 * par.degree - 1]

    @staticmethod
    def expansion_exponents(par: BfvParameters, level: int) -> List[int]:
        """evaluation_key.rs:349-351: (N >> l) + 1 for l < level."""
        return [(par.degree >> l) + 1 for l in range(level)]

    def add_keys(self, sk: SecretKey, exponents: Sequence[int], rng: np.random.Generator):
        for e in exponents:
            if e not in self.gk:
                self.gk[e] = GaloisKey(sk, e, self.ciphertext_level, self.evaluation_key_level, rng)

    def computes_inner_sum(self, ct: Ciphertext) -> Ciphertext:
        """evaluation_key.rs:56-83."""
        out = ct.copy()
        for e in self.inner_sum_exponents(self.par):
            out = out + self.gk[e].relinearize(out)
        return out

    def monomial(self, l: int) -> Poly:
        """evaluation_key.rs:355-363: -x^(N - 2^l) in the ciphertext context, Ntt."""
        n = self.par.degree
        v = np.zeros(n, dtype=np.int64)
        v[n - (1 << l)] = -1
        return Poly.from_i64(self.par.context_at_level(self.ciphertext_level), v).into_ntt()

    def expands(self, ct: Ciphertext, size: int) -> List[Ciphertext]:
        """evaluation_key.rs:148-193 (oblivious expansion, eprint 2019/1483)."""
        level = max(size - 1, 0).bit_length()
        out = [ct.copy()] + [None] * ((1 << level) - 1)
        for l in range(level):
            mono = self.monomial(l)
            gk = self.gk[(self.par.degree >> l) + 1]
            step = 1 << l
            for i in range(step):
                sub = gk.relinearize(out[i])
                j = step | i
                if j < size:
                    t = Ciphertext(self.par, [a - b for a, b in zip(out[i].c, sub.c)], out[i].level)
                    out[j] = Ciphertext(self.par, [c * mono for c in t.c], t.level)
                out[i] = out[i] + sub
        return out[:size]

    def rotates_columns_by(self, ct: Ciphertext, i: int) -> Ciphertext:
        return self.gk[self.rot_to_gk_exponent[i]].relinearize(ct)


class Multiplicator:
    """ops/mul.rs:21-227 `Multiplicator`."""

    def __init__(self, lhs: ScalingFactor, rhs: ScalingFactor, extended_basis: Sequence[int],
                 post: ScalingFactor, level: int, par: BfvParameters):
        self.par = par
        self.level = level
        self.base_ctx = par.context_at_level(level)
        self.mul_ctx = Context(list(extended_basis), par.degree)
        self.extender_lhs = Scaler(self.base_ctx, self.mul_ctx, lhs)
        self.extender_rhs = Scaler(self.base_ctx, self.mul_ctx, rhs)
        self.down_scaler = Scaler(self.mul_ctx, self.base_ctx, post)
        self.rk: Optional[RelinearizationKey] = None
        self.mod_switch = False

    @staticmethod
    def default_extended_basis(par: BfvParameters, level: int) -> List[int]:
        """mul.rs:102-117."""
        ctx = par.context_at_level(level)
        modulus_size = sum(par.moduli_sizes[:len(ctx.moduli)])
        n_moduli = (modulus_size + 60 + 61) // 62
        ext = list(ctx.moduli)
        ub = 1 << 62
        while len(ext) != len(ctx.moduli) + n_moduli:
            ub = generate_prime(62, 2 * par.degree, ub)
            if ub not in ext and ub not in ctx.moduli:
                ext.append(ub)
        return ext

    @staticmethod
    def default(rk: RelinearizationKey) -> "Multiplicator":
        """mul.rs:101-130."""
        par, level = rk.ksk.par, rk.ksk.ciphertext_level
        ctx = par.context_at_level(level)
        m = Multiplicator(ScalingFactor.one(), ScalingFactor.one(), Multiplicator.default_extended_basis(par, level),
                          ScalingFactor(par.plaintext, ctx.modulus()), level, par)
        m.enable_relinearization(rk)
        return m

    def enable_relinearization(self, rk: RelinearizationKey):
        if self.par.context_at_level(rk.ksk.ciphertext_level) != self.base_ctx:
            raise ValueError("Invalid relinearization key context")
        self.rk = rk

    def enable_mod_switching(self):
        if self.par.context_at_level(self.par.max_level()) == self.base_ctx:
            raise ValueError("Cannot modulo switch as this is already the last level")
        self.mod_switch = True

    def multiply(self, lhs: Ciphertext, rhs: Ciphertext) -> Ciphertext:
        """mul.rs:158-227."""
        if lhs.level != self.level or rhs.level != self.level:
            raise ValueError("Ciphertexts are not at expected level")
        if len(lhs) != 2 or len(rhs) != 2:
            raise ValueError("Multiplication can only be performed on ciphertexts of size 2")
        c00 = lhs[0].scale(self.extender_lhs)
        c01 = lhs[1].scale(self.extender_lhs)
        c10 = rhs[0].scale(self.extender_rhs)
        c11 = rhs[1].scale(self.extender_rhs)
        c0 = c00 * c10
        c1 = c00 * c11
        c1 += c01 * c10
        c2 = c01 * c11
        c = [c0.scale(self.down_scaler), c1.scale(self.down_scaler), c2.scale(self.down_scaler)]
        if self.rk is not None:
            c2_pb = c[2].copy().into_power_basis()
            c0r, c1r = self.rk.relinearizes_poly(c2_pb)
            if c0r.ctx != c[0].ctx:
                c0r = c0r.into_power_basis().switch_down_to(c[0].ctx).into_ntt()
                c1r = c1r.into_power_basis().switch_down_to(c[1].ctx).into_ntt()
            c[0] += c0r
            c[1] += c1r
            c = c[:2]
        out = Ciphertext(self.par, c, self.level)
        if self.mod_switch:
            out.switch_down()
        return out


def _ctx_desc(ctx: Context, keep: list) -> OraCtx:
    """The tables of a context for oracle.cpp's whole-product loop."""
    n = ctx.degree
    mods = _u64(np.concatenate([q.fields for q in ctx.q]))
    ptrs = []
    for name in ("omegas", "omegas_shoup", "zetas_inv", "zetas_inv_shoup"):
        arr = (U64P * len(ctx.ops))(*[_p(getattr(op, name)) for op in ctx.ops])
        ptrs.append(arr)
    sinv = _u64([op.size_inv for op in ctx.ops])
    sinv_s = _u64([op.size_inv_shoup for op in ctx.ops])
    keep += [mods, sinv, sinv_s] + ptrs
    return OraCtx(len(ctx.moduli), n, _p(mods), ptrs[0], ptrs[1], ptrs[2], ptrs[3], _p(sinv), _p(sinv_s))


class MultiplyDriver:
    """ops/mul.rs:158-227 `Multiplicator::multiply` run whole in oracle.cpp
    over independent pairs on host threads: the timed CPU baseline. Covers the
    default multiplicator (relinearization key at the multiplication level, no
    modulus switching); outputs equal `Multiplicator.multiply`."""

    def __init__(self, m: "Multiplicator"):
        if m.rk is None or m.mod_switch or m.rk.ksk.ctx_ksk != m.base_ctx:
            raise ValueError("the driver runs the default multiplicator only")
        self.m = m
        self._keep = []
        k = m.rk.ksk
        self.c0 = np.ascontiguousarray(np.stack([p.coefficients for p in k.c0]))
        self.c0s = np.ascontiguousarray(np.stack([p.coefficients_shoup for p in k.c0]))
        self.c1 = np.ascontiguousarray(np.stack([p.coefficients for p in k.c1]))
        self.c1s = np.ascontiguousarray(np.stack([p.coefficients_shoup for p in k.c1]))
        self.desc = OraMult(
            _ctx_desc(m.base_ctx, self._keep), _ctx_desc(m.mul_ctx, self._keep),
            ctypes.pointer(m.extender_lhs.scaler._desc), m.extender_lhs.number_common_moduli,
            ctypes.pointer(m.extender_rhs.scaler._desc), m.extender_rhs.number_common_moduli,
            ctypes.pointer(m.down_scaler.scaler._desc), _p(self.c0), _p(self.c0s), _p(self.c1), _p(self.c1s))

    def multiply(self, lhs: np.ndarray, rhs: np.ndarray, threads: int = 1) -> np.ndarray:
        """lhs, rhs [count][2][L][N] (Ntt) -> [count][2][L][N]."""
        lhs = np.ascontiguousarray(lhs, dtype=np.uint64)
        rhs = np.ascontiguousarray(rhs, dtype=np.uint64)
        assert lhs.shape == rhs.shape and lhs.shape[1:] == (2, len(self.m.base_ctx.moduli), self.m.base_ctx.degree)
        out = np.zeros_like(lhs)
        lib().ora_multiply(ctypes.byref(self.desc), _p(lhs), _p(rhs), _p(out), lhs.shape[0], threads)
        return out


def dot_product_scalar(cts: Sequence[Ciphertext], pts: Sequence[Poly]) -> Ciphertext:
    """ops/dot_product.rs:56-140: sum_i ct_i * pt_i (pt_i the plaintexts' Ntt
    polynomials), accumulated exactly and reduced once per coefficient."""
    first = cts[0]
    parts = []
    for k in range(len(first)):
        acc = None
        for ct, pt in zip(cts, pts):
            prod = ct[k].coefficients.astype(object) * pt.coefficients.astype(object)
            acc = prod if acc is None else acc + prod
        q = np.array(first[k].ctx.moduli, dtype=object)[:, None]
        c = (acc % q).astype(np.uint64)
        parts.append(Poly(first[k].ctx, c, NTT))
    return Ciphertext(first.par, parts, first.level)


# ---------------------------------------------------------------------------
# fhe-util/src/lib.rs:57-135 transcoding and the Rq coefficient payload
# (fhe-math/src/rq/convert.rs:17-42, 44-93; zq/mod.rs:783-793).


def transcode_to_bytes(a: Sequence[int], nbits: int) -> bytes:
    """lib.rs:57-95: little-endian bit packing of nbits-bit values."""
    assert 0 < nbits <= 64
    mask = (1 << nbits) - 1
    acc, acc_bits, out = 0, 0, bytearray()
    for v in a:
        acc |= (int(v) & mask) << acc_bits
        acc_bits += nbits
        while acc_bits >= 8:
            out.append(acc & 0xFF)
            acc >>= 8
            acc_bits -= 8
    if acc_bits > 0:
        out.append(acc & 0xFF)
    return bytes(out)


def transcode_from_bytes(b: bytes, nbits: int) -> List[int]:
    """lib.rs:97-135."""
    assert 0 < nbits <= 64
    mask = (1 << nbits) - 1
    acc, acc_bits, out = 0, 0, []
    for byte in b:
        acc |= int(byte) << acc_bits
        acc_bits += 8
        while acc_bits >= nbits:
            out.append(acc & mask)
            acc >>= nbits
            acc_bits -= nbits
    if acc_bits > 0:
        out.append(acc)
    return out


def modulus_nbits(p: int) -> int:
    """zq/mod.rs:783-786: bits of p - 1."""
    return (p - 1).bit_length()


def rq_payload(p: "Poly") -> bytes:
    """convert.rs:17-42: power-basis coefficients of every limb, each packed
    with the bit length of its modulus, concatenated."""
    q = p.copy()
    if q.representation != POWER_BASIS:
        q.into_power_basis()
    return b"".join(transcode_to_bytes(q.coefficients[i].tolist(), modulus_nbits(m))
                    for i, m in enumerate(q.ctx.moduli))


def rq_from_payload(ctx: Context, payload: bytes, representation: str) -> "Poly":
    """convert.rs:44-93 + TryConvertFrom<&Rq>: unpack every limb (values
    reduced modulo the limb's modulus), then back to `representation`."""
    n = ctx.degree
    rows, index = [], 0
    for m in ctx.moduli:
        size = (n * modulus_nbits(m) + 7) // 8
        vals = transcode_from_bytes(payload[index:index + size], modulus_nbits(m))[:n]
        rows.append(np.array([v % m for v in vals], dtype=np.uint64))
        index += size
    p = Poly(ctx, np.stack(rows), POWER_BASIS)
    if representation != POWER_BASIS:
        p.into_ntt()
    return p


# ---------------------------------------------------------------------------
# Protobuf framing (prost 0.14 encoding of rq.proto / bfv.proto): fields in
# tag order, proto3 defaults (0, false, empty) omitted, every element of a
# repeated bytes field written. Restated from the published wire format:
# varints of 7 bits per byte (low groups first), keys (field << 3) | type,
# type 0 = varint, 2 = length-delimited.

REPRESENTATION_CODE = {POWER_BASIS: 1, NTT: 2, NTT_SHOUP: 3}


def _varint(v: int) -> bytes:
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _pb_varint(field: int, v: int) -> bytes:
    return b"" if v == 0 else _varint(field << 3) + _varint(v)


def _pb_bytes(field: int, b: bytes, repeated: bool = False) -> bytes:
    if not b and not repeated:
        return b""
    return _varint((field << 3) | 2) + _varint(len(b)) + bytes(b)


def rq_message(p: "Poly", allow_variable_time: bool = False) -> bytes:
    """rq/convert.rs:17-42 (`Rq::from(&Poly)`) then `encode_to_vec`."""
    return (_pb_varint(1, REPRESENTATION_CODE[p.representation]) + _pb_varint(2, p.ctx.degree) +
            _pb_bytes(3, rq_payload(p)) + _pb_varint(4, int(allow_variable_time)))


def ciphertext_message(ct: "Ciphertext", seed: Optional[bytes] = None, allow_variable_time: bool = False) -> bytes:
    """fhe/src/bfv/ciphertext.rs:164-191: every part but the last as an Rq
    message, the last one too unless the ciphertext carries its seed."""
    polys = ct.c[:-1] if seed else ct.c
    out = b"".join(_pb_bytes(1, rq_message(p, allow_variable_time), repeated=True) for p in polys)
    if seed:
        out += _pb_bytes(2, seed)
    return out + _pb_varint(3, ct.level)


def parse_fields(b: bytes) -> List[tuple]:
    """(field, wire type, value) of a message: ints for varints, bytes for
    length-delimited fields (fixed32 / fixed64 values as bytes)."""
    out, i = [], 0

    def varint():
        nonlocal i
        v, shift = 0, 0
        while True:
            if i >= len(b) or shift > 63:
                raise ValueError("truncated varint")
            c = b[i]
            i += 1
            v |= (c & 0x7F) << shift
            shift += 7
            if not c & 0x80:
                return v

    while i < len(b):
        key = varint()
        field, wt = key >> 3, key & 7
        if wt == 0:
            out.append((field, wt, varint()))
        elif wt == 2:
            n = varint()
            if i + n > len(b):
                raise ValueError("truncated field")
            out.append((field, wt, bytes(b[i:i + n])))
            i += n
        elif wt == 1:
            out.append((field, wt, bytes(b[i:i + 8])))
            i += 8
        elif wt == 5:
            out.append((field, wt, bytes(b[i:i + 4])))
            i += 4
        else:
            raise ValueError("unsupported wire type")
    return out


def ciphertext_from_message(par: "BfvParameters", b: bytes) -> "Ciphertext":
    """fhe/src/bfv/ciphertext.rs:195-240 `TryConvertFrom<&CiphertextProto>`."""
    cs, seed, level = [], b"", 0
    for f, wt, v in parse_fields(b):
        if f == 1 and wt == 2:
            cs.append(v)
        elif f == 2 and wt == 2:
            seed = v
        elif f == 3 and wt == 0:
            level = v & 0xFFFFFFFF
    if not cs or (len(cs) == 1 and not seed):
        raise ValueError("Not enough polynomials")
    if level > par.max_level():
        raise ValueError("InvalidLevel")
    ctx = par.context_at_level(level)
    polys = []
    for m in cs:
        rep, degree, coeffs = 0, 0, b""
        for f, wt, v in parse_fields(m):
            if f == 1 and wt == 0:
                rep = v
            elif f == 2 and wt == 0:
                degree = v
            elif f == 3 and wt == 2:
                coeffs = v
        if rep != REPRESENTATION_CODE[NTT]:
            raise ValueError("representation")
        if degree != ctx.degree or len(coeffs) != sum((degree * modulus_nbits(q) + 7) // 8 for q in ctx.moduli):
            raise ValueError("Invalid coefficients")
        polys.append(rq_from_payload(ctx, coeffs, NTT))
    if seed:
        if len(seed) != 32:
            raise ValueError("InvalidSeedSize")
        polys.append(Poly(ctx, random_from_seed(ctx, seed), NTT))
    return Ciphertext(par, polys, level)


def ksk_message(ksk: "KeySwitchingKey", allow_variable_time: bool = True) -> bytes:
    """fhe/src/bfv/keys/key_switching_key.rs:332-352: c0[i] (and c1[i] unless
    the key has its seed) as NttShoup Rq messages, the seed, the levels and
    the decomposition base (0 for RNS-digit keys)."""
    seed = getattr(ksk, "seed", None)
    out = b"".join(_pb_bytes(1, rq_message(p, allow_variable_time), repeated=True) for p in ksk.c0)
    if seed is None:
        out += b"".join(_pb_bytes(2, rq_message(p, allow_variable_time), repeated=True) for p in ksk.c1)
    else:
        out += _pb_bytes(3, seed)
    return (out + _pb_varint(4, ksk.ciphertext_level) + _pb_varint(5, ksk.ksk_level)
            + _pb_varint(6, getattr(ksk, "log_base", 0)))


def relinearization_key_message(rk: "RelinearizationKey") -> bytes:
    """relinearization_key.rs:109-115: { ksk = 1 }."""
    return _pb_bytes(1, ksk_message(rk.ksk), repeated=True)


def galois_key_message(gk: "GaloisKey") -> bytes:
    """galois_key.rs:127-134: { ksk = 1, exponent = 2 }."""
    return _pb_bytes(1, ksk_message(gk.ksk), repeated=True) + _pb_varint(2, gk.element.exponent)


def evaluation_key_message(gks: Sequence["GaloisKey"], ciphertext_level: int, evaluation_key_level: int) -> bytes:
    """evaluation_key.rs:382-392: { repeated GaloisKey gk = 2; ciphertext_level
    = 3; evaluation_key_level = 4 }, the keys in the order given."""
    return (b"".join(_pb_bytes(2, galois_key_message(g), repeated=True) for g in gks)
            + _pb_varint(3, ciphertext_level) + _pb_varint(4, evaluation_key_level))
