"""Seeded polynomials on the GPU (Poly::random_from_seed, rq/mod.rs:239-257):
bit-exact against the oracle's SHA-256 + ChaCha8 + Uniform restatement,
including moduli that reject draws often (the exact walk), seeded
ciphertexts (ciphertext.rs:220-237) and seeded key-switching keys
(key_switching_key.rs:108-123, 383-406)."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


def _seeds(rng, count):
    return [bytes(rng.integers(0, 256, 32, dtype=np.uint8)) for _ in range(count)]


def _dev_seeds(fg, seeds):
    import torch
    return torch.tensor(np.frombuffer(b"".join(seeds), dtype=np.uint8).reshape(-1, 32), device="cuda")


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 2), (16384, 6), (32768, 3)])
def test_random_from_seed_matches_oracle(fg, ora, cuda, n, L):
    par = ora.BfvParameters(n, 65537 if n > 16 else 1153, moduli_sizes=[62] * L)
    ctx_o = ora.Context(par.moduli, n)
    ctx = fg.Context(par.moduli, n)
    seeds = _seeds(np.random.default_rng(n + L), 3) + [bytes(32)]
    got = fg.to_host(fg.random_from_seed(ctx, _dev_seeds(fg, seeds)))
    for b, sd in enumerate(seeds):
        assert np.array_equal(got[b], ora.random_from_seed(ctx_o, sd)), b


def test_random_from_seed_rejections(fg, ora, cuda):
    """Moduli just above 2^61 reject about one draw in eight: every polynomial
    takes the exact walk, and limbs start after the previous limb's last draw."""
    n = 1024
    moduli, ub = [], (1 << 61) + (1 << 50)
    while len(moduli) < 3:
        ub = ora.generate_prime(62, 2 * n, ub)
        moduli.append(ub)
    assert all(ora.uniform_u64_threshold(q) > (1 << 58) for q in moduli)
    ctx_o, ctx = ora.Context(moduli, n), fg.Context(moduli, n)
    seeds = _seeds(np.random.default_rng(5), 4)
    got = fg.to_host(fg.random_from_seed(ctx, _dev_seeds(fg, seeds)))
    for b, sd in enumerate(seeds):
        assert np.array_equal(got[b], ora.random_from_seed(ctx_o, sd)), b


@pytest.mark.parametrize("n,variance", [(16, 10), (4096, 10), (16384, 16), (8, 1), (1000, 7), (4096, 3)])
def test_sample_cbd_from_seed_matches_oracle(fg, ora, cuda, n, variance):
    """sample_vec_cbd (fhe-util/src/lib.rs:22-55) over ChaCha8Rng::from_seed
    streams: each vector equals the oracle's (n = 1000 leaves a partial last
    chunk of 16 samples; variance 16 takes whole 64-bit draws per sample)."""
    seeds = _seeds(np.random.default_rng(n * variance), 3) + [bytes(32)]
    got = fg.to_host(fg.sample_cbd_from_seed(_dev_seeds(fg, seeds), variance, n)).view(np.int64)
    assert got.shape == (4, n)
    for b, sd in enumerate(seeds):
        assert np.array_equal(got[b], ora.sample_vec_cbd_from_seed(n, variance, sd)), b


def test_sample_cbd_errors(fg, cuda):
    seeds = _dev_seeds(fg, [bytes(32)])
    for v in (0, 17):
        with pytest.raises(fg.FhegError) as e:
            fg.sample_cbd_from_seed(seeds, v, 16)
        assert e.value.code == fg.ERR_INVALID_ARGUMENT


def test_encrypt_from_seeds(fg, ora, cuda):
    """SecretKey::try_encrypt (secret_key.rs:102-138) entirely on the device:
    a from its seed (Poly::random_from_seed), e from the caller's
    ChaCha8Rng::from_seed (Poly::small), b = e - a s + m; equal to the
    oracle's ciphertext for the same seeds, and it decrypts."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=31)
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    ctx_o = s.par_o.context_at_level(0)
    ctx = fg.Context(ctx_o.moduli, 4096)
    a_seeds, e_seeds = _seeds(s.rng, 3), _seeds(s.rng, 3)
    vals = s.rng.integers(0, 65537, (3, 4096), dtype=np.uint64)
    a = fg.random_from_seed(ctx, _dev_seeds(fg, a_seeds))
    e = fg.sample_cbd_from_seed(_dev_seeds(fg, e_seeds), s.par_o.variance, 4096)
    got = fg.to_host(sk.encrypt(fg.to_device(vals), a, e, 0, simd=True))
    for b in range(3):
        pt = ora.Plaintext.encode(vals[b], "simd", s.par_o, 0)
        want = s.sk.encrypt_with(pt, ora.random_from_seed(ctx_o, a_seeds[b]),
                                 ora.sample_vec_cbd_from_seed(4096, s.par_o.variance, e_seeds[b]))
        assert np.array_equal(got[b], want.to_array()), b
    dec = fg.to_host(sk.decrypt(fg.to_device(got), 0, simd=True))
    assert np.array_equal(dec, vals)


def test_seeded_ciphertexts(fg, ora, cuda):
    """A fresh ciphertext sent as (c0, seed): c1 expanded on the device into a
    [count][2][L][N] batch in place, equal to the oracle's, and the batch
    decrypts on the device."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=21)
    ctx_o = s.par_o.context_at_level(0)
    seeds = _seeds(s.rng, 3)
    vals, cts = [], []
    for sd in seeds:
        v = s.rng.integers(0, 65537, 4096, dtype=np.uint64)
        a = ora.random_from_seed(ctx_o, sd)
        e = ora.sample_vec_cbd(4096, s.par_o.variance, s.rng)
        cts.append(s.sk.encrypt_with(ora.Plaintext.encode(v, "simd", s.par_o), a, e).to_array())
        vals.append(v)
    want = np.stack(cts)
    batch = np.zeros_like(want)
    batch[:, 0] = want[:, 0]
    dev = fg.to_device(batch)
    ctx = s.par.context_at_level(0)
    fg.random_from_seed(ctx, _dev_seeds(fg, seeds), out=dev[:, 1], poly_stride=2 * 3 * 4096)
    assert np.array_equal(fg.to_host(dev), want)
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    assert np.array_equal(fg.to_host(sk.decrypt(dev, 0)), np.stack(vals))


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 3)])
def test_seeded_keys(fg, ora, cuda, n, L):
    """Relinearization and Galois keys uploaded as (c0, seed) give the same
    results as the keys uploaded whole."""
    s = Setup(fg, ora, n, L, 65537 if n > 16 else 1153, seed=n + 31)
    seed = bytes(range(1, 33))
    rk_o = ora.RelinearizationKey(s.sk, s.rng, seed=seed)
    assert rk_o.ksk.c1_array().shape == (L, L, n)
    rk = fg.RelinearizationKey.from_seed(s.par, rk_o.ksk.c0_array(), seed)
    _, cts = s.encrypt(2)
    mo = ora.Multiplicator.default(ora.RelinearizationKey.from_ksk(rk_o.ksk))
    prod = fg.Multiplicator.default(rk).multiply(fg.to_device(cts[0].to_array()[None]),
                                                 fg.to_device(cts[1].to_array()[None]))
    assert np.array_equal(fg.to_host(prod)[0], mo.multiply(cts[0], cts[1]).to_array())
    e = 2 * n - 1
    gk_o = ora.GaloisKey(s.sk, e, 0, 0, s.rng, seed=seed[::-1])
    gk = fg.GaloisKey.from_seed(s.par, e, gk_o.ksk.c0_array(), seed[::-1])
    got = fg.to_host(gk.relinearize(fg.to_device(cts[0].to_array()[None])))[0]
    assert np.array_equal(got, gk_o.relinearize(cts[0]).to_array())
    with pytest.raises(fg.FhegError):
        fg.RelinearizationKey.from_seed(s.par, rk_o.ksk.c0_array(), b"short")
