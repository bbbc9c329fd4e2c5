"""Ciphertext messages on the GPU path (bfv.proto Ciphertext of rq.proto Rq
parts, fhe/src/bfv/ciphertext.rs:164-240, fhe-math/src/rq/convert.rs:17-135):
the bytes equal the oracle's prost-equivalent encoding, decoding gives the
oracle's polynomials, seeded messages expand their last part on the device,
and malformed messages fail with the reference's error kinds."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,L,t", [(16, 3, 1153), (4096, 3, 65537), (16384, 6, 65537)])
def test_ciphertext_bytes_match_oracle(fg, ora, cuda, n, L, t):
    s = Setup(fg, ora, n, L, t, seed=3 * n + L)
    for level in (0, 1):
        ctx = s.par_o.context_at_level(level)
        _, cts = s.encrypt(3, level=level)
        seeds = [bytes(s.rng.integers(0, 256, 32, dtype=np.uint8)) for _ in cts]
        for b, sd in enumerate(seeds):
            cts[b].c[1] = ora.Poly(ctx, ora.random_from_seed(ctx, sd), ora.NTT)
        dev = fg.to_device(np.stack([c.to_array() for c in cts]))
        for seeded in (False, True):
            for avt in (False, True):
                got = fg.ciphertext_to_bytes(s.par, level, dev, seeds if seeded else None, avt)
                for b, c in enumerate(cts):
                    assert got[b] == ora.ciphertext_message(c, seeds[b] if seeded else None, avt), (level, b)
                assert fg.ciphertext_peek(s.par, got[0]) == (level, 2, seeded)
                back = fg.to_host(fg.ciphertext_from_bytes(s.par, got))
                assert np.array_equal(back, fg.to_host(dev)), (level, seeded, avt)


def test_three_part_and_oracle_messages(fg, ora, cuda):
    """Messages written by the oracle decode on the device, including a 3-part
    (unrelinearized) product at level 1."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=77)
    vals, cts = s.encrypt(2, level=1)
    ext = ora.Multiplicator.default_extended_basis(s.par_o, 1)
    q = s.par_o.context_at_level(1).modulus()
    mo3 = ora.Multiplicator(ora.ScalingFactor.one(), ora.ScalingFactor.one(), ext, ora.ScalingFactor(65537, q), 1,
                            s.par_o)
    prod = mo3.multiply(cts[0], cts[1])
    msg = ora.ciphertext_message(prod)
    assert fg.ciphertext_peek(s.par, msg) == (1, 3, False)
    got = fg.to_host(fg.ciphertext_from_bytes(s.par, [msg, msg]))
    assert np.array_equal(got[1], prod.to_array())
    assert fg.ciphertext_to_bytes(s.par, 1, fg.to_device(prod.to_array()[None]))[0] == msg
    # Unknown fields are skipped, fields may come in any order.
    reordered = ora._pb_varint(3, 1) + ora._pb_varint(9, 5) + msg[:msg.rfind(b"\x18")]
    assert np.array_equal(fg.to_host(fg.ciphertext_from_bytes(s.par, [reordered]))[0], prod.to_array())


def test_ciphertext_bytes_errors(fg, ora, cuda):
    s = Setup(fg, ora, 16, 3, 1153, seed=5)
    _, cts = s.encrypt(1)
    ct = cts[0]
    good = ora.ciphertext_message(ct)

    def code(msg, batch=None):
        with pytest.raises(fg.FhegError) as e:
            if batch is None:
                fg.ciphertext_peek(s.par, msg)
                fg.ciphertext_from_bytes(s.par, [msg])
            else:
                fg.ciphertext_from_bytes(s.par, batch)
        return e.value.code

    rq = ora.rq_message(ct[0])
    assert code(ora._pb_bytes(1, rq, repeated=True)) == fg.ERR_WRONG_PARTS  # one part, no seed
    assert code(b"") == fg.ERR_WRONG_PARTS
    assert code(good + ora._pb_varint(3, 7)) == fg.ERR_INVALID_LEVEL
    assert code(ora._pb_bytes(1, rq, repeated=True) + ora._pb_bytes(2, bytes(31))) == fg.ERR_INVALID_ARGUMENT
    assert code(good[:-3]) == fg.ERR_INVALID_ARGUMENT  # truncated
    pb = ct[0].copy().into_power_basis()
    bad_rep = ora._pb_bytes(1, ora.rq_message(pb), repeated=True) * 2
    assert code(bad_rep) == fg.ERR_INVALID_ARGUMENT
    no_rep = ora._pb_bytes(1, rq[2:], repeated=True) * 2  # representation field dropped: Unknown
    assert code(no_rep) == fg.ERR_INVALID_ARGUMENT
    bad_deg = ora._pb_bytes(1, b"\x08\x02\x10\x20" + rq[4:], repeated=True) * 2  # degree 32
    assert code(bad_deg) == fg.ERR_INVALID_ARGUMENT
    short = ora._pb_bytes(1, ora._pb_varint(1, 2) + ora._pb_varint(2, 16) + ora._pb_bytes(3, bytes(10)),
                          repeated=True) * 2
    assert code(short) == fg.ERR_INVALID_ARGUMENT
    seeded = ora.ciphertext_message(ct, bytes(32))
    assert code(None, batch=[good, seeded]) == fg.ERR_INVALID_ARGUMENT  # mixed batch


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 3)])
def test_key_messages(fg, ora, cuda, n, L):
    """RelinearizationKey / GaloisKey / KeySwitchingKey::from_bytes
    (key_switching_key.rs:354-420): keys decoded on the device from the
    reference's messages, seeded or not, give the oracle's results."""
    s = Setup(fg, ora, n, L, 65537 if n > 16 else 1153, seed=n + 7)
    _, cts = s.encrypt(2)
    lhs, rhs = (fg.to_device(c.to_array()[None]) for c in cts)
    for seed in (None, bytes(range(5, 37))):
        rk_o = ora.RelinearizationKey(s.sk, s.rng, seed=seed)
        rk = fg.RelinearizationKey.from_bytes(s.par, ora.relinearization_key_message(rk_o))
        assert (rk.ciphertext_level, rk.ksk_level) == (0, 0)
        want = ora.Multiplicator.default(rk_o).multiply(cts[0], cts[1]).to_array()
        assert np.array_equal(fg.to_host(fg.Multiplicator.default(rk).multiply(lhs, rhs))[0], want)
        e = pow(3, 2, 2 * n)
        gk_o = ora.GaloisKey(s.sk, e, 0, 0, s.rng, seed=seed)
        gk = fg.GaloisKey.from_bytes(s.par, ora.galois_key_message(gk_o))
        assert gk.exponent == e
        got = fg.to_host(gk.relinearize(lhs))[0]
        assert np.array_equal(got, gk_o.relinearize(cts[0]).to_array())
        ksk = fg.KeySwitchingKey.from_bytes(s.par, ora.ksk_message(gk_o.ksk))
        assert (ksk.ciphertext_level, ksk.ksk_level) == (0, 0)


def test_key_message_errors(fg, ora, cuda):
    s = Setup(fg, ora, 16, 3, 1153, seed=8)
    gk_o = ora.GaloisKey(s.sk, 3, 0, 0, s.rng, seed=bytes(32))
    k = gk_o.ksk
    c0 = b"".join(ora._pb_bytes(1, ora.rq_message(p, True), repeated=True) for p in k.c0)
    tail = ora._pb_bytes(3, bytes(32))

    def code(msg, cls=fg.KeySwitchingKey):
        with pytest.raises(fg.FhegError) as e:
            cls.from_bytes(s.par, msg)
        return e.value.code

    assert code(c0[:len(c0) * 2 // 3] + tail) == fg.ERR_INVALID_ARGUMENT  # too few c0 / truncated
    assert code(c0 + ora._pb_bytes(3, bytes(31))) == fg.ERR_INVALID_ARGUMENT  # seed length
    assert code(c0) == fg.ERR_INVALID_ARGUMENT  # no c1 and no seed
    assert code(c0 + tail + ora._pb_varint(4, 9)) == fg.ERR_INVALID_LEVEL
    assert code(c0 + tail + ora._pb_varint(6, 30)) == fg.ERR_INVALID_ARGUMENT  # decomposition base, levels not maximal
    ntt = b"".join(ora._pb_bytes(1, ora.rq_message(ora.Poly(p.ctx, p.coefficients, ora.NTT)), repeated=True)
                   for p in k.c0)
    assert code(ntt + tail) == fg.ERR_INVALID_ARGUMENT  # Ntt instead of NttShoup
    assert code(b"", fg.RelinearizationKey) == fg.ERR_INVALID_ARGUMENT  # no ksk field
    even = ora._pb_bytes(1, ora.ksk_message(k), repeated=True) + ora._pb_varint(2, 4)
    assert code(even, fg.GaloisKey) == fg.ERR_INVALID_ARGUMENT
    ok = fg.GaloisKey.from_bytes(s.par, ora.galois_key_message(gk_o))
    assert ok.exponent == 3


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 3)])
def test_key_to_bytes_and_evaluation_key(fg, ora, cuda, n, L):
    """KeySwitchingKey / RelinearizationKey / GaloisKey::to_bytes from device
    keys (key_switching_key.rs:332-352) equal the reference's messages, seeded
    or not and with a decomposition base; EvaluationKey messages
    (evaluation_key.rs:382-432) decode into working keys and encode back."""
    s = Setup(fg, ora, n, L, 65537 if n > 16 else 1153, seed=n + 9)
    for seed in (None, bytes(range(9, 41))):
        rk_o = ora.RelinearizationKey(s.sk, s.rng, seed=seed)
        msg = ora.relinearization_key_message(rk_o)
        if seed:
            rk = fg.RelinearizationKey.from_seed(s.par, rk_o.ksk.c0_array(), seed)
        else:
            rk = fg.RelinearizationKey(s.par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array())
        assert rk.to_bytes() == msg
        assert fg.RelinearizationKey.from_bytes(s.par, msg).to_bytes() == msg
        gk_o = ora.GaloisKey(s.sk, 2 * n - 1, 1, 0, s.rng, seed=seed)
        gmsg = ora.galois_key_message(gk_o)
        assert fg.GaloisKey.from_bytes(s.par, gmsg).to_bytes() == gmsg
        assert fg.KeySwitchingKey.from_bytes(s.par, ora.ksk_message(gk_o.ksk)).to_bytes() == ora.ksk_message(gk_o.ksk)
    last = L - 1
    dk_o = ora.GaloisKey(s.sk, 3, last, last, s.rng)
    dk = fg.GaloisKey(s.par, 3, dk_o.ksk.c0_array(), dk_o.ksk.c1_array(), last, last)
    assert dk.to_bytes() == ora.galois_key_message(dk_o)
    # EvaluationKey at (ciphertext level 1, key level 0).
    gks_o = [ora.GaloisKey(s.sk, ora.rotation_exponent(s.par_o, i), 1, 0, s.rng, seed=bytes([i]) * 32)
             for i in (1, 2)] + [ora.GaloisKey(s.sk, 2 * n - 1, 1, 0, s.rng)]
    emsg = ora.evaluation_key_message(gks_o, 1, 0)
    keys, cl, el = fg.evaluation_key_from_bytes(s.par, emsg)
    assert (cl, el) == (1, 0) and [k.exponent for k in keys] == [g.element.exponent for g in gks_o]
    _, cts = s.encrypt(1, level=1)
    ct = fg.to_device(cts[0].to_array()[None])
    for k, g in zip(keys, gks_o):
        assert np.array_equal(fg.to_host(k.relinearize(ct))[0], g.relinearize(cts[0]).to_array())
    assert fg.evaluation_key_to_bytes(keys, 1, 0) == emsg
    with pytest.raises(fg.FhegError) as e:  # a key at other levels than the message names
        fg.evaluation_key_from_bytes(s.par, ora.evaluation_key_message(gks_o, 1, 1))
    assert e.value.code == fg.ERR_INVALID_ARGUMENT
