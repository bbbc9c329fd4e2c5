"""Key levels. Keys below the ciphertext level (more moduli than the
ciphertext): the key switch runs in the key's context and its output is
switched down to the ciphertext's context before the additions, as the
reference does (relinearization_key.rs:84-92, galois_key.rs:113-120,
ops/mul.rs:199-206, rq/mod.rs:455-462). Keys at the last level (one modulus):
the key switch decomposes its input in base 2^31 instead of by residues
(key_switching_key.rs:63-89, 172-211, 292-329). Every path is compared bit
for bit with the oracle and decrypted."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


def _rk(fg, ora, s, ct_level, key_level):
    rk_o = ora.RelinearizationKey(s.sk, s.rng, ct_level, key_level)
    rk = fg.RelinearizationKey(s.par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), ct_level, key_level)
    return rk_o, rk


def _gk(fg, ora, s, e, ct_level, key_level):
    gk_o = ora.GaloisKey(s.sk, e, ct_level, key_level, s.rng)
    gk = fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), ct_level, key_level)
    return gk_o, gk


@pytest.mark.parametrize("n,L,ct_level,key_level,B", [(16384, 6, 2, 0, 2), (32768, 12, 5, 0, 1),
                                                      (4096, 5, 3, 1, 3), (16, 4, 2, 0, 2)])
def test_multiply_with_lower_level_key(fg, ora, cuda, n, L, ct_level, key_level, B):
    t = 65537 if n > 16 else 1153
    s = Setup(fg, ora, n, L, t, seed=7000 + n + ct_level, level=ct_level)
    rk_o, rk = _rk(fg, ora, s, ct_level, key_level)
    mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    vals, cts = s.encrypt(2 * B)
    lhs = np.stack([c.to_array() for c in cts[:B]])
    rhs = np.stack([c.to_array() for c in cts[B:]])
    out = fg.to_host(mult.multiply(fg.to_device(lhs), fg.to_device(rhs)))
    assert out.shape == (B, 2, L - ct_level, n)
    for b in range(B):
        want = mult_o.multiply(cts[b], cts[B + b])
        assert np.array_equal(out[b], want.to_array()), f"pair {b}"
        assert list(s.decrypt(out[b], ct_level)) == s.product(vals[b], vals[B + b])


def test_multiply_with_lower_level_key_every_plan(fg, ora, cuda):
    """The switched-down relinearization under both stage-F forms and a
    two-pass plan, and with modulus switching after it."""
    s = Setup(fg, ora, 16384, 4, 65537, seed=7100, level=1)
    rk_o, rk = _rk(fg, ora, s, 1, 0)
    m = fg.Multiplicator.default(rk)
    m.set_small_plan(0)
    vals, cts = s.encrypt(4)
    lhs = fg.to_device(np.stack([cts[0].to_array(), cts[1].to_array()]))
    rhs = fg.to_device(np.stack([cts[2].to_array(), cts[3].to_array()]))
    mo = ora.Multiplicator.default(rk_o)
    want = np.stack([mo.multiply(cts[0], cts[2]).to_array(), mo.multiply(cts[1], cts[3]).to_array()])
    for plan in ([14, 14, 14, 14, 0, 0], [14, 14, 14, 14, 1, 0], [12, 12, 12, 12, 0, 0], [13, 12, 14, 12, 1, 1]):
        m.plan = plan
        assert np.array_equal(fg.to_host(m.multiply(lhs, rhs)), want), plan
    mo.enable_mod_switching()
    m.enable_mod_switching()
    out = fg.to_host(m.multiply(lhs, rhs))
    for b in range(2):
        w = mo.multiply(cts[b], cts[2 + b])
        assert w.level == 2 and np.array_equal(out[b], w.to_array())
        assert list(s.decrypt(out[b], 2)) == s.product(vals[b], vals[2 + b])


@pytest.mark.parametrize("n,L,ct_level,key_level", [(16384, 6, 2, 0), (4096, 4, 2, 1)])
def test_relinearize_with_lower_level_key(fg, ora, cuda, n, L, ct_level, key_level):
    s = Setup(fg, ora, n, L, 65537, seed=7200 + n, level=ct_level)
    rk_o, rk = _rk(fg, ora, s, ct_level, key_level)
    vals, cts = s.encrypt(4)
    prods = [cts[0] * cts[1], cts[2] * cts[3]]
    ct3 = fg.to_device(np.stack([p.to_array() for p in prods]))
    out = fg.to_host(rk.relinearizes(ct3))
    for b in range(2):
        want = rk_o.relinearizes(prods[b])
        assert np.array_equal(out[b], want.to_array()), b
        assert list(s.decrypt(out[b], ct_level)) == s.product(vals[2 * b], vals[2 * b + 1])


@pytest.mark.parametrize("n,L,ct_level,key_level", [(32768, 12, 5, 0), (4096, 5, 3, 1)])
def test_rotation_with_lower_level_key(fg, ora, cuda, n, L, ct_level, key_level):
    s = Setup(fg, ora, n, L, 65537, seed=7300 + n, level=ct_level)
    e = ora.rotation_exponent(s.par_o, 3)
    gk_o, gk = _gk(fg, ora, s, e, ct_level, key_level)
    vals, cts = s.encrypt(2)
    out = fg.to_host(gk.relinearize(fg.to_device(np.stack([c.to_array() for c in cts]))))
    half = n // 2
    for b in range(2):
        assert np.array_equal(out[b], gk_o.relinearize(cts[b]).to_array()), b
        want = np.concatenate([np.roll(vals[b][:half], -3), np.roll(vals[b][half:], -3)])
        assert np.array_equal(s.decrypt(out[b], ct_level), want)


@pytest.mark.parametrize("count", [7, 18])
def test_ragged_batch_mixing_key_levels(fg, ora, cuda, count):
    """One ragged batch with same-level keys and keys one to four levels below
    the ciphertext (18 requests run as two concurrent halves)."""
    n, L = 4096, 6
    s = Setup(fg, ora, n, L, 65537, seed=7400 + count)
    rng = np.random.default_rng(count)
    keys, cts_d, want = [], [], []
    for b in range(count):
        ct_level = int(rng.integers(0, L - 1))
        key_level = ct_level if b % 3 == 0 else int(rng.integers(0, ct_level + 1))
        e = ora.rotation_exponent(s.par_o, int(rng.integers(1, n // 2))) if b % 2 else 2 * n - 1
        gk_o, gk = _gk(fg, ora, s, e, ct_level, key_level)
        keys.append(gk)
        _, cts = s.encrypt(1, level=ct_level)
        cts_d.append(fg.to_device(cts[0].to_array()))
        want.append(gk_o.relinearize(cts[0]).to_array())
    outs = fg.rotate_batch(s.par, keys, cts_d)
    for b in range(count):
        assert np.array_equal(fg.to_host(outs[b]), want[b]), f"entry {b}"


def test_server_with_lower_level_keys(fg, ora, cuda):
    """mul+relin and rotations whose keys lie below the ciphertext level,
    submitted together to one server."""
    s = Setup(fg, ora, 16384, 5, 65537, seed=7500, level=2)
    rk_o, rk = _rk(fg, ora, s, 2, 0)
    mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    gk_o, gk = _gk(fg, ora, s, 2 * 16384 - 1, 2, 1)
    _, cts = s.encrypt(6)
    with fg.Server(hbm_budget_bytes=2 << 30, streams=2, max_batch=8) as srv:
        ids = [srv.submit_mul_relin(mult, cts[0].to_array(), cts[1].to_array()),
               srv.submit_rotate(gk, cts[2].to_array()),
               srv.submit_mul_relin(mult, cts[3].to_array(), cts[4].to_array()),
               srv.submit_rotate(gk, cts[5].to_array())]
        got = [srv.wait(r) for r in ids]
    assert np.array_equal(got[0], mult_o.multiply(cts[0], cts[1]).to_array())
    assert np.array_equal(got[1], gk_o.relinearize(cts[2]).to_array())
    assert np.array_equal(got[2], mult_o.multiply(cts[3], cts[4]).to_array())
    assert np.array_equal(got[3], gk_o.relinearize(cts[5]).to_array())


def _decomp_relin_key(fg, ora, s, level):
    """A relinearization key at the last level: the reference builds such a
    key from bytes only (RelinearizationKey::new refuses one modulus), so the
    oracle's key is assembled from its KeySwitchingKey."""
    ctx = s.par_o.context_at_level(level)
    sk_ntt = s.sk.s_ntt(ctx)
    ksk = ora.KeySwitchingKey(s.sk, (sk_ntt * sk_ntt).into_power_basis(), level, level, s.rng)
    assert ksk.log_base == 31 and len(ksk.c0) == 2
    rk_o = ora.RelinearizationKey.from_ksk(ksk)
    return rk_o, fg.RelinearizationKey(s.par, ksk.c0_array(), ksk.c1_array(), level, level)


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 3), (16384, 2)])
def test_decomposition_rotation_relin_and_multiply(fg, ora, cuda, n, L):
    t = 65537 if n > 16 else 1153
    last = L - 1
    s = Setup(fg, ora, n, L, t, seed=7600 + n, level=last)
    e = ora.rotation_exponent(s.par_o, 1)
    gk_o, gk = _gk(fg, ora, s, e, last, last)
    assert gk_o.ksk.log_base == 31
    vals, cts = s.encrypt(4)
    batch = fg.to_device(np.stack([c.to_array() for c in cts]))
    rot = fg.to_host(gk.relinearize(batch))
    half = n // 2
    for b in range(4):
        assert np.array_equal(rot[b], gk_o.relinearize(cts[b]).to_array()), b
        want = np.concatenate([np.roll(vals[b][:half], -1), np.roll(vals[b][half:], -1)])
        assert np.array_equal(s.decrypt(rot[b], last), want)
    rk_o, rk = _decomp_relin_key(fg, ora, s, last)
    prods = [cts[0] * cts[1], cts[2] * cts[3]]
    out = fg.to_host(rk.relinearizes(fg.to_device(np.stack([p.to_array() for p in prods]))))
    for b in range(2):
        assert np.array_equal(out[b], rk_o.relinearizes(prods[b]).to_array()), b
    mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    got = fg.to_host(mult.multiply(batch[:2].contiguous(), batch[2:].contiguous()))
    for b in range(2):
        want = mult_o.multiply(cts[b], cts[2 + b])
        assert np.array_equal(got[b], want.to_array()), b
        assert list(s.decrypt(got[b], last)) == s.product(vals[b], vals[2 + b])


def test_decomposition_in_ragged_batch_and_key_messages(fg, ora, cuda):
    """Decomposition keys next to RNS-digit keys in one ragged batch, and
    Galois key messages carrying the base (key_switching_key.rs:332-372)."""
    n, L = 4096, 4
    s = Setup(fg, ora, n, L, 65537, seed=7700)
    keys, cts_d, want = [], [], []
    for b, (ct_level, key_level) in enumerate([(3, 3), (1, 1), (3, 3), (2, 0), (0, 0), (3, 3)]):
        e = ora.rotation_exponent(s.par_o, 1 + b)
        gk_o = ora.GaloisKey(s.sk, e, ct_level, key_level, s.rng, seed=bytes([b]) * 32 if b % 2 else None)
        if b < 3:
            gk = fg.GaloisKey.from_bytes(s.par, ora.galois_key_message(gk_o))
            assert (gk.exponent, gk.ciphertext_level, gk.ksk_level) == (e, ct_level, key_level)
        else:
            gk = fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), ct_level, key_level)
        keys.append(gk)
        _, cts = s.encrypt(1, level=ct_level)
        cts_d.append(fg.to_device(cts[0].to_array()))
        want.append(gk_o.relinearize(cts[0]).to_array())
    outs = fg.rotate_batch(s.par, keys, cts_d)
    for b in range(len(keys)):
        assert np.array_equal(fg.to_host(outs[b]), want[b]), f"entry {b}"
