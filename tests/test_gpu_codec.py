"""Plaintext side on the GPU: SIMD and coefficient encoding into the
plaintext's Ntt polynomial, ciphertext x plaintext products, decryption with
decoding, bit-exact against the oracle."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,L,t", [(16, 3, 1153), (4096, 2, 65537), (16384, 6, 65537), (32768, 4, 65537)])
def test_encode_matches_oracle(fg, ora, cuda, n, L, t):
    s = Setup(fg, ora, n, L, t, seed=7 * n + L)
    rng = np.random.default_rng(n)
    vals = rng.integers(0, t, (3, n), dtype=np.uint64)
    for level in (0, L - 1):
        ctx = s.par_o.context_at_level(level)
        for enc in ("simd", "poly"):
            got = fg.to_host(fg.plaintext_encode(s.par, level, fg.to_device(vals), simd=enc == "simd"))
            for b in range(3):
                v = ora.Plaintext.encode(vals[b], enc, s.par_o, level).value
                want = ora.Poly.from_u64(ctx, v).into_ntt().coefficients
                assert np.array_equal(got[b], want), (level, enc, b)


@pytest.mark.parametrize("n,L,t", [(16, 3, 1153), (4096, 3, 65537), (16384, 6, 65537), (32768, 4, 65537)])
def test_decrypt_matches_oracle(fg, ora, cuda, n, L, t):
    s = Setup(fg, ora, n, L, t, seed=11 * n + L)
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    for level in (0, L - 1):
        vals, cts = s.encrypt(3, level=level)
        arr = fg.to_device(np.stack([c.to_array() for c in cts]))
        got = fg.to_host(sk.decrypt(arr, level))
        for b in range(3):
            assert [int(x) for x in got[b]] == [int(x) for x in vals[b]], (level, b)
        raw = fg.to_host(sk.decrypt(arr, level, simd=False))
        for b in range(3):
            assert np.array_equal(raw[b], s.sk.decrypt(cts[b]).value), (level, b)


def test_decrypt_three_parts(fg, ora, cuda):
    """The phase c0 + c1 s + c2 s^2 of an unrelinearized product."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=3)
    vals, cts = s.encrypt(2)
    ext = ora.Multiplicator.default_extended_basis(s.par_o, 0)
    q = s.par_o.context_at_level(0).modulus()
    mo3 = ora.Multiplicator(ora.ScalingFactor.one(), ora.ScalingFactor.one(), ext, ora.ScalingFactor(65537, q), 0,
                            s.par_o)
    prod = mo3.multiply(cts[0], cts[1]).to_array()
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    got = fg.to_host(sk.decrypt(fg.to_device(prod[None])))[0]
    assert [int(x) for x in got] == s.product(vals[0], vals[1])


@pytest.mark.parametrize("n,L", [(4096, 2), (16384, 6)])
def test_mul_plain(fg, ora, cuda, n, L):
    """ct x pt (ops/mod.rs:229-238): bit-exact per part, decrypts to the slotwise product."""
    s = Setup(fg, ora, n, L, 65537, seed=n + 5)
    vals, cts = s.encrypt(3)
    pv = np.random.default_rng(2).integers(0, 65537, (3, n), dtype=np.uint64)
    pt = fg.plaintext_encode(s.par, 0, fg.to_device(pv))
    ct = fg.to_device(np.stack([c.to_array() for c in cts]))
    got = fg.to_host(fg.ciphertext_mul_plain(s.par, 0, ct, pt))
    shared = fg.to_host(fg.ciphertext_mul_plain(s.par, 0, ct, pt[0]))
    ctx = s.par_o.context_at_level(0)
    for b in range(3):
        m = ora.Poly.from_u64(ctx, ora.Plaintext.encode(pv[b], "simd", s.par_o).value).into_ntt()
        want = np.stack([(cts[b][k] * m).coefficients for k in range(2)])
        assert np.array_equal(got[b], want)
        assert list(s.decrypt(got[b], 0)) == s.product(vals[b], pv[b])
        assert list(s.decrypt(shared[b], 0)) == s.product(vals[b], pv[0])


@pytest.mark.parametrize("n,L,t", [(16, 3, 1153), (4096, 3, 65537), (16384, 6, 65537)])
def test_encrypt_matches_oracle(fg, ora, cuda, n, L, t):
    """try_encrypt with the randomness given (secret_key.rs:102-138): the
    device ciphertext equals the oracle's for the same a and e, and decrypts."""
    s = Setup(fg, ora, n, L, t, seed=13 * n + L)
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    for level in (0, L - 1):
        ctx = s.par_o.context_at_level(level)
        vals = s.rng.integers(0, t, (3, n), dtype=np.uint64)
        a = np.stack([ora.Poly.random(ctx, ora.NTT, s.rng).coefficients for _ in range(3)])
        e = np.stack([ora.sample_vec_cbd(n, s.par_o.variance, s.rng) for _ in range(3)]).astype(np.int64)
        for enc in ("simd", "poly"):
            got = fg.to_host(sk.encrypt(fg.to_device(vals), fg.to_device(a), fg.to_device(e.view(np.uint64)),
                                        level, simd=enc == "simd"))
            for b in range(3):
                pt = ora.Plaintext.encode(vals[b], enc, s.par_o, level)
                want = s.sk.encrypt_with(pt, a[b], e[b])
                assert np.array_equal(got[b], want.to_array()), (level, enc, b)
            dec = fg.to_host(sk.decrypt(fg.to_device(got), level, simd=enc == "simd"))
            assert np.array_equal(dec, vals), (level, enc)
