"""Pins the CPU oracle to the reference's own known answers and exact-formula
tests (fhe-math), restated here. No GPU involved."""

import numpy as np
import pytest


def test_nfl_62bit_primes(ora):
    """fhe-math/src/zq/primes.rs:67-102: the only literal golden vector."""
    expected = [
        4611686018326724609, 4611686018309947393, 4611686018282684417, 4611686018257518593,
        4611686018232352769, 4611686018171535361, 4611686018106523649, 4611686018058289153,
        4611686018051997697, 4611686017974403073, 4611686017812922369, 4611686017781465089,
        4611686017773076481, 4611686017678704641, 4611686017666121729, 4611686017647247361,
        4611686017590624257, 4611686017554972673, 4611686017529806849, 4611686017517223937,
    ]
    generated, ub = [], ((1 << 64) - 1) >> 2
    while len(generated) != 20:
        p = ora.generate_prime(62, 2 * 1048576, ub)
        assert p is not None
        ub = p
        generated.append(p)
    assert generated == expected


def test_generate_prime_edges(ora):
    """primes.rs:104-122."""
    assert ora.generate_prime(10, 2048, 1 << 10) is None
    assert ora.generate_prime(11, 16, 1033) is None


def test_ntt_constructor(ora):
    """ntt/mod.rs:30-49."""
    for size in (32, 1024):
        for p in (1153, 4611686018326724609):
            ok = ora.supports_ntt(p, size)
            if ok:
                ora.NttOperator(ora.Modulus(p), size)
            else:
                with pytest.raises(ValueError):
                    ora.NttOperator(ora.Modulus(p), size)
    assert ora.supports_ntt(1153, 32) and not ora.supports_ntt(1153, 1024)


@pytest.mark.parametrize("size,p", [(32, 1153), (32, 4611686018326724609), (1024, 4611686018326724609)])
def test_ntt_bijection_and_lazy(ora, size, p):
    """ntt/mod.rs:51-112: forward/backward bijection, lazy == reduced."""
    rng = np.random.default_rng(size + p % 1000)
    op = ora.NttOperator(ora.Modulus(p), size)
    for _ in range(20):
        a = rng.integers(0, p, size, dtype=np.uint64)
        b = a.copy()
        op.forward(b)
        assert not np.array_equal(a, b)
        lazy = a.copy()
        op.forward_vt_lazy(lazy)
        assert (lazy < np.uint64(4 * p)).all()
        op.p.reduce_vec(lazy)
        assert np.array_equal(lazy, b)
        op.backward(b)
        assert np.array_equal(a, b)


def test_ntt_is_evaluation_at_odd_powers(ora):
    """The forward NTT evaluates the polynomial at psi^(2*bitrev(i)+1)."""
    p, n = 4611686018326724609, 64
    op = ora.NttOperator(ora.Modulus(p), n)
    rng = np.random.default_rng(3)
    a = rng.integers(0, p, n, dtype=np.uint64)
    b = a.copy()
    op.forward(b)
    for i in range(n):
        e = 2 * ora.bitrev(i, 6) + 1
        want = sum(int(a[j]) * pow(op.omega, e * j, p) for j in range(n)) % p
        assert int(b[i]) == want


def _expected_scaled(x, q_mod, t_mod, n, d):
    """rns/scaler.rs:397-414: centered rounding of x * n / d."""
    sign = x >= (q_mod >> 1)
    if sign:
        x = q_mod - x
        if d % 2 == 0:
            return t_mod - ((x * n + ((d >> 1) - 1)) // d) % t_mod
        return t_mod - ((x * n + (d >> 1)) // d) % t_mod
    return (x * n + (d >> 1)) // d


NUMS = [1, 2, 3, 100, 1000, 4611686018326724610]
DENS = [1, 2, 3, 4, 100, 101, 1000, 1001, 4611686018326724610]


def test_rns_scaler_same_context(ora):
    """rns/scaler.rs:379-419."""
    rng = np.random.default_rng(11)
    q = ora.RnsContext([4, 4611686018326724609, 1153])
    for n in NUMS:
        for d in DENS:
            s = ora.RnsScaler(q, q, ora.ScalingFactor(n, d))
            for _ in range(40):
                x = [int(rng.integers(0, m)) for m in q.moduli_u64]
                lift = q.lift(x)
                z = s.scale_new(x, len(x))
                assert z == q.project(_expected_scaled(lift, q.modulus(), q.modulus(), n, d))


def test_rns_scaler_different_contexts(ora):
    """rns/scaler.rs:421-473."""
    rng = np.random.default_rng(12)
    q = ora.RnsContext([4, 4611686018326724609, 1153])
    r = ora.RnsContext([4, 4611686018326724609, 1153, 4611686018309947393, 4611686018282684417,
                        4611686018257518593, 4611686018232352769, 4611686018171535361, 4611686018106523649,
                        4611686018058289153])
    for n in NUMS:
        for d in DENS:
            s = ora.RnsScaler(q, r, ora.ScalingFactor(n, d))
            for _ in range(20):
                x = [int(rng.integers(0, m)) for m in q.moduli_u64]
                lift = q.lift(x)
                y = s.scale_new(x, len(r.moduli))
                assert y == r.project(_expected_scaled(lift, q.modulus(), r.modulus(), n, d))


RQ_Q = [4611686018282684417, 4611686018326724609, 4611686018309947393]
RQ_P = [4611686018282684417, 4611686018309947393, 4611686018257518593]


def test_rq_scaler(ora):
    """rq/scaler.rs:152-203 (power basis and Ntt give the same result)."""
    rng = np.random.default_rng(13)
    frm, to = ora.Context(RQ_Q, 16), ora.Context(RQ_P, 16)
    for n in NUMS:
        for d in DENS:
            sc = ora.Scaler(frm, to, ora.ScalingFactor(n, d))
            for _ in range(3):
                p = ora.Poly.random(frm, ora.POWER_BASIS, rng)
                expected = [_expected_scaled(x, frm.modulus(), to.modulus(), n, d) % to.modulus()
                            for x in p.to_biguints()]
                assert sc.scale(p).to_biguints() == expected
                pn = p.copy().into_ntt()
                assert sc.scale(pn).into_power_basis().to_biguints() == expected


MODULI = [1153, 4611686018326724609, 4611686018309947393, 4611686018232352769, 4611686018171535361]


def test_switch_down_formula(ora):
    """rq/mod.rs:984-1017: switch_down = round(x * Q' / Q)."""
    rng = np.random.default_rng(14)
    ctx = ora.Context(MODULI, 16)
    for _ in range(10):
        p = ora.Poly.random(ctx, ora.POWER_BASIS, rng)
        reference = p.to_biguints()
        cur = ctx
        while cur.next_context is not None:
            den = cur.modulus()
            cur = cur.next_context
            num = cur.modulus()
            p.switch_down()
            got = p.to_biguints()
            assert got == [((b * num) + (den >> 1)) // den % cur.modulus() for b in reference]
            reference = got


def test_substitute_identities(ora):
    """rq/mod.rs:892-982."""
    rng = np.random.default_rng(15)
    for m in MODULI:
        ctx = ora.Context([m], 16)
        p = ora.Poly.random(ctx, ora.POWER_BASIS, rng)
        p_ntt = p.copy().into_ntt()
        for e in (0, 2, 16):
            with pytest.raises(ValueError):
                ora.SubstitutionExponent(ctx, e)
        e1, e3, e11 = (ora.SubstitutionExponent(ctx, k) for k in (1, 3, 11))
        assert np.array_equal(p.substitute(e1).coefficients, p.coefficients)
        assert np.array_equal(p_ntt.substitute(e1).coefficients, p_ntt.coefficients)
        q = p.substitute(e3)
        v = np.zeros(16, dtype=np.uint64)
        pc = p.coefficients[0]
        for i in range(16):
            v[(3 * i) % 16] = m - pc[i] if ((3 * i) // 16) & 1 == 1 and pc[i] > 0 else pc[i]
        assert np.array_equal(q.coefficients[0], v)
        assert np.array_equal(p_ntt.substitute(e3).coefficients, q.copy().into_ntt().coefficients)
        assert np.array_equal(p.substitute(e3).substitute(e11).coefficients, p.coefficients)
        assert np.array_equal(p_ntt.substitute(e3).substitute(e11).coefficients, p_ntt.coefficients)


def test_lazy_constant_ntt(ora):
    """rq/mod.rs:823-848: lazy reduction then `forward_vt_lazy` of a row."""
    m = MODULI[0]
    ctx = ora.Context([m], 16)
    coeffs = np.array([(i * m + i) % (1 << 64) for i in range(16)], dtype=np.uint64)
    digits = np.ascontiguousarray(coeffs[None, :])
    expected = coeffs.copy()
    ctx.q[0].lazy_reduce_vec(expected)
    ctx.ops[0].forward_vt_lazy(expected)
    got = digits.copy()
    ctx.q[0].lazy_reduce_vec(got[0])
    ctx.ops[0].forward_vt_lazy(got[0])
    assert np.array_equal(got[0], expected)


@pytest.mark.parametrize("L", [3, 6])
def test_multiplicator_decrypts(ora, L):
    """ops/mul.rs:246-339 (N=16, t=1153): product decrypts to the slotwise
    product, with and without relinearization and mod switching."""
    rng = np.random.default_rng(100 + L)
    par = ora.BfvParameters(16, 1153, moduli_sizes=[62] * L)
    for _ in range(3):
        values = rng.integers(0, 1153, 16, dtype=np.uint64)
        expected = (values.astype(object) * values.astype(object)) % 1153
        sk = ora.SecretKey.random(par, rng)
        rk = ora.RelinearizationKey(sk, rng)
        pt = ora.Plaintext.encode(values, "simd", par)
        ct1, ct2 = sk.encrypt(pt, rng), sk.encrypt(pt, rng)
        m = ora.Multiplicator.default(rk)
        ct3 = m.multiply(ct1, ct2)
        assert list(sk.decrypt(ct3).decode("simd")) == list(expected)
        m.rk = None
        ct3 = m.multiply(ct1, ct2)
        assert len(ct3) == 3
        assert list(sk.decrypt(ct3).decode("simd")) == list(expected)
        m.enable_relinearization(rk)
        m.enable_mod_switching()
        ct3 = m.multiply(ct1, ct2)
        assert ct3.level == 1
        assert list(sk.decrypt(ct3).decode("simd")) == list(expected)


def test_key_switch_decomposition(ora):
    """key_switching_key.rs:529-561 (default_arc(6, 16), level 5: a single
    modulus, so the key switches by base-2^31 digits): c0 + c1 s - input * p
    stays within half the modulus' bits plus 10 (the same bound)."""
    rng = np.random.default_rng(530)
    par = ora.BfvParameters(16, 1153, moduli_sizes=[62] * 6)
    ctx = par.context_at_level(5)
    for _ in range(20):
        sk = ora.SecretKey.random(par, rng)
        p = ora.Poly.small(ctx, ora.POWER_BASIS, 10, rng)
        ksk = ora.KeySwitchingKey(sk, p, 5, 5, rng)
        assert ksk.log_base == 31 and len(ksk.c0) == 2
        s = sk.s_ntt(ctx)
        inp = ora.Poly.random(ctx, ora.POWER_BASIS, rng)
        c0, c1 = ksk.key_switch(inp)
        c2 = (c0 + c1 * s).into_power_basis()
        c3 = (inp.copy().into_ntt() * p.copy().into_ntt()).into_power_basis()
        q = ctx.modulus()
        for b in (c2 - c3).to_biguints():
            assert min(b.bit_length(), (q - b).bit_length()) <= q.bit_length() // 2 + 10


@pytest.mark.parametrize("n,L,threads", [(16, 3, 1), (4096, 2, 3), (8192, 3, 2)])
def test_multiply_driver_equals_orchestrated_oracle(ora, n, L, threads):
    """The whole-product C++ loop of the timed CPU baseline (ops/mul.rs:158-227
    on host threads) equals the orchestrated oracle Multiplicator, product by
    product."""
    t = 1153 if n == 16 else 65537
    rng = np.random.default_rng(n + L)
    par = ora.BfvParameters(n, t, moduli_sizes=[62] * L)
    sk = ora.SecretKey.random(par, rng)
    m = ora.Multiplicator.default(ora.RelinearizationKey(sk, rng))
    cts = [sk.encrypt(ora.Plaintext.encode(rng.integers(0, t, n, dtype=np.uint64), "simd", par), rng)
           for _ in range(6)]
    lhs = np.stack([c.to_array() for c in cts[:3]])
    rhs = np.stack([c.to_array() for c in cts[3:]])
    got = ora.MultiplyDriver(m).multiply(lhs, rhs, threads)
    for k in range(3):
        assert np.array_equal(got[k], m.multiply(cts[k], cts[3 + k]).to_array()), k


@pytest.mark.parametrize("L", [2, 8])
def test_rgsw_external_product_decrypts(ora, L):
    """rgsw_ciphertext.rs:172-210 (default_arc(2, 16) and (8, 16)): ct1 x
    RGSW(pt2) decrypts to the same plaintext as the 3-part product ct1 * ct2."""
    rng = np.random.default_rng(300 + L)
    par = ora.BfvParameters(16, 1153, moduli_sizes=[62] * L)
    sk = ora.SecretKey.random(par, rng)
    v1 = rng.integers(0, 1153, 16, dtype=np.uint64)
    v2 = rng.integers(0, 1153, 16, dtype=np.uint64)
    pt1, pt2 = ora.Plaintext.encode(v1, "simd", par), ora.Plaintext.encode(v2, "simd", par)
    ct1, ct2 = sk.encrypt(pt1, rng), sk.encrypt(pt2, rng)
    rgsw = ora.RGSWCiphertext(sk, pt2, rng)
    expected = sk.decrypt(ct1 * ct2).decode("simd")
    assert list(expected) == [int(a) * int(b) % 1153 for a, b in zip(v1, v2)]
    ct3 = rgsw.external_product(ct1)
    assert np.array_equal(sk.decrypt(ct3).decode("simd"), expected)


def test_rotations_decrypt(ora):
    """evaluation_key.rs:572-675: row and column rotations."""
    rng = np.random.default_rng(7)
    n = 16
    par = ora.BfvParameters(n, 1153, moduli_sizes=[62] * 3)
    sk = ora.SecretKey.random(par, rng)
    ek = ora.EvaluationKey(sk, rng, columns=range(1, n // 2), row_rotation=True)
    values = rng.integers(0, 1153, n, dtype=np.uint64)
    ct = sk.encrypt(ora.Plaintext.encode(values, "simd", par), rng)
    half = n // 2
    for i in range(1, half):
        got = sk.decrypt(ek.rotates_columns_by(ct, i)).decode("simd")
        want = np.concatenate([np.roll(values[:half], -i), np.roll(values[half:], -i)])
        assert np.array_equal(got, want)
    got = sk.decrypt(ek.rotates_rows(ct)).decode("simd")
    assert np.array_equal(got, np.concatenate([values[half:], values[:half]]))


def test_transcode_known_and_roundtrip(ora):
    """fhe-util/src/lib.rs:255-304: the known round trip, the empty case and
    self-consistency for every width."""
    b = ora.transcode_to_bytes([1, 2, 3, 4], 4)
    assert b == bytes([0x21, 0x43])
    assert ora.transcode_from_bytes(b, 4)[:4] == [1, 2, 3, 4]
    assert ora.transcode_to_bytes([], 8) == b"" and ora.transcode_from_bytes(b"", 8) == []
    rng = np.random.default_rng(3)
    for size in (1, 7, 33):
        vals = [int(x) for x in rng.integers(0, 2**63, size, dtype=np.uint64)]
        for nbits in (1, 5, 17, 31, 62, 63):
            masked = [v & ((1 << nbits) - 1) for v in vals]
            bb = ora.transcode_to_bytes(masked, nbits)
            assert len(bb) == (size * nbits + 7) // 8
            assert ora.transcode_from_bytes(bb, nbits)[:size] == masked


def test_rq_payload_roundtrip(ora):
    """rq/serialize.rs tests: power basis and Ntt survive the payload."""
    rng = np.random.default_rng(4)
    moduli = [4611686018282684417, 4611686018326724609, 4611686018309947393]
    ctx = ora.Context(moduli, 16)
    c = np.stack([rng.integers(0, m, 16, dtype=np.uint64) for m in moduli])
    for rep in (ora.POWER_BASIS, ora.NTT):
        p = ora.Poly(ctx, c.copy(), rep)
        payload = ora.rq_payload(p)
        assert len(payload) == 3 * 16 * 62 // 8
        assert np.array_equal(ora.rq_from_payload(ctx, payload, rep).coefficients, c)


def test_chacha_block_function(ora):
    """The vectorised block function equals the scalar generator's stream, and
    at 20 rounds equals ChaCha20 of the `cryptography` package (OpenSSL) with
    the 16-byte counter-and-nonce block set to (64-bit counter, 64-bit stream),
    the rand_chacha state layout."""
    key = [(0x01234567 * (i + 1)) & 0xFFFFFFFF for i in range(8)]
    rng = ora.ChaChaRng(key)
    words = [rng.next_u32() for _ in range(16 * 5)]
    assert list(ora.chacha_blocks(key, np.arange(5)).reshape(-1)) == words
    draws = ora.chacha_u64_draws(key, 3, 30)
    rng = ora.ChaChaRng(key)
    ref = [rng.next_u64() for _ in range(33)][3:]
    assert [int(x) for x in draws] == ref
    ciphers = pytest.importorskip("cryptography.hazmat.primitives.ciphers")
    kb = b"".join(w.to_bytes(4, "little") for w in key)
    for counter, stream in [(0, 0), (7, 0), (3, 0x1122334455667788)]:
        nonce = counter.to_bytes(8, "little") + stream.to_bytes(8, "little")
        enc = ciphers.Cipher(ciphers.algorithms.ChaCha20(kb, nonce), mode=None).encryptor()
        ks = enc.update(bytes(64 * 2))
        got = ora.chacha_blocks(key, np.array([counter, counter + 1]), rounds=20, stream=stream)
        assert got.astype("<u4").tobytes() == ks


def _cbd_pool(size, variance, next_u64):
    """fhe-util/src/lib.rs:22-55 step by step: a bit pool refilled with a
    64-bit draw above the bits it holds whenever fewer than 4v remain."""
    nb = 4 * variance
    mask_add = ((2**64 - 1) >> (64 - nb)) >> (2 * variance)
    mask_sub = mask_add << (2 * variance)
    pool, nbits, out = 0, 0, []
    for _ in range(size):
        if nbits < nb:
            pool |= next_u64() << nbits
            nbits += 64
        out.append(bin(pool & mask_add).count("1") - bin(pool & mask_sub).count("1"))
        pool >>= nb
        nbits -= nb
    return out, nbits


@pytest.mark.parametrize("size,variance", [(1, 1), (7, 3), (100, 10), (64, 16), (33, 5), (16, 16), (50, 2)])
def test_cbd_from_seed_is_the_pool_algorithm(ora, size, variance):
    """The oracle's CBD over a ChaCha8Rng::from_seed stream (cutting the
    draws' bit stream into 4v-bit samples) equals the reference's pool
    algorithm run on ChaChaRng.from_seed draws, and both take
    ceil(4 v size / 64) draws."""
    seed = bytes((7 * i + size) & 0xFF for i in range(32))
    rng = ora.ChaChaRng.from_seed(seed)
    draws = []

    def next_u64():
        draws.append(rng.next_u64())
        return draws[-1]

    want, _ = _cbd_pool(size, variance, next_u64)
    assert len(draws) == (4 * variance * size + 63) // 64
    got = ora.sample_vec_cbd_from_seed(size, variance, seed)
    assert [int(x) for x in got] == want
    assert all(abs(x) <= 2 * variance for x in want)
    with pytest.raises(ValueError):
        ora.sample_vec_cbd_from_seed(size, 17, seed)


def test_random_from_seed(ora):
    """rq/mod.rs:239-257 and key_switching_key.rs:108-123: deterministic in
    the seed, uniform residues, seeds of c1 drawn 32 bytes at a time, and the
    exact rejection walk (a modulus just above 2^61 rejects about one draw in
    eight, and every limb then starts after the last accepted draw)."""
    ctx = ora.Context(ora.BfvParameters(16, 1153, moduli_sizes=[62] * 3).moduli, 16)
    seed = bytes(range(32))
    a = ora.random_from_seed(ctx, seed)
    assert np.array_equal(a, ora.random_from_seed(ctx, seed))
    assert not np.array_equal(a, ora.random_from_seed(ctx, bytes(32)))
    for j, q in enumerate(ctx.moduli):
        assert int(a[j].max()) < q
    digest = __import__("hashlib").sha256(seed).digest()
    key = [int.from_bytes(digest[4 * i:4 * i + 4], "little") for i in range(8)]
    # Near-2^62 moduli reject with probability ~2^-46: no rejections here.
    draws = ora.chacha_u64_draws(key, 0, 48)
    want = [(int(x) * ctx.moduli[k // 16]) >> 64 for k, x in enumerate(draws)]
    assert [int(v) for v in a.reshape(-1)] == want
    # generate_c1: seed i = bytes 32 i .. 32 i + 31 of the key seed's stream.
    rng = ora.ChaChaRng.from_seed(seed)
    stream = rng.fill_bytes(96)
    assert ora.ksk_c1_seeds(seed, 3) == [stream[0:32], stream[32:64], stream[64:96]]
    # A modulus just above 2^61 (threshold ~ 2^61 - 7 delta): sequential walk.
    q = ora.generate_prime(62, 32, (1 << 61) + (1 << 45))
    assert q is not None and q > (1 << 61)
    ctx2 = ora.Context([q, ctx.moduli[0]], 16)
    b = ora.random_from_seed(ctx2, seed)
    thresh = ora.uniform_u64_threshold(q)
    draws = [int(x) for x in ora.chacha_u64_draws(key, 0, 200)]
    vals, pos = [], 0
    while len(vals) < 16:
        prod = draws[pos] * q
        pos += 1
        if prod & ora.M64 >= thresh:
            vals.append(prod >> 64)
    assert pos > 16, "expected at least one rejection"
    assert [int(v) for v in b[0]] == vals
    vals = [(draws[pos + k] * ctx.moduli[0]) >> 64 for k in range(16)]
    assert [int(v) for v in b[1]] == vals


def _proto_classes():
    """rq.proto Rq and bfv.proto Ciphertext as dynamic message classes of the
    `protobuf` package (no protoc needed)."""
    descriptor_pb2 = pytest.importorskip("google.protobuf.descriptor_pb2")
    from google.protobuf import descriptor_pool, message_factory
    F = descriptor_pb2.FieldDescriptorProto
    fd = descriptor_pb2.FileDescriptorProto(name="fheg_wire_pin.proto", package="pin", syntax="proto3")
    enum = fd.enum_type.add(name="Representation")
    for name, num in [("UNKNOWN", 0), ("POWERBASIS", 1), ("NTT", 2), ("NTTSHOUP", 3)]:
        enum.value.add(name=name, number=num)
    rq = fd.message_type.add(name="Rq")
    rq.field.add(name="representation", number=1, type=F.TYPE_ENUM, type_name=".pin.Representation",
                 label=F.LABEL_OPTIONAL)
    rq.field.add(name="degree", number=2, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    rq.field.add(name="coefficients", number=3, type=F.TYPE_BYTES, label=F.LABEL_OPTIONAL)
    rq.field.add(name="allow_variable_time", number=4, type=F.TYPE_BOOL, label=F.LABEL_OPTIONAL)
    ct = fd.message_type.add(name="Ciphertext")
    ct.field.add(name="c", number=1, type=F.TYPE_BYTES, label=F.LABEL_REPEATED)
    ct.field.add(name="seed", number=2, type=F.TYPE_BYTES, label=F.LABEL_OPTIONAL)
    ct.field.add(name="level", number=3, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    ksk = fd.message_type.add(name="KeySwitchingKey")
    ksk.field.add(name="c0", number=1, type=F.TYPE_BYTES, label=F.LABEL_REPEATED)
    ksk.field.add(name="c1", number=2, type=F.TYPE_BYTES, label=F.LABEL_REPEATED)
    ksk.field.add(name="seed", number=3, type=F.TYPE_BYTES, label=F.LABEL_OPTIONAL)
    for name, num in [("ciphertext_level", 4), ("ksk_level", 5), ("log_base", 6)]:
        ksk.field.add(name=name, number=num, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    gk = fd.message_type.add(name="GaloisKey")
    gk.field.add(name="ksk", number=1, type=F.TYPE_MESSAGE, type_name=".pin.KeySwitchingKey", label=F.LABEL_OPTIONAL)
    gk.field.add(name="exponent", number=2, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    ek = fd.message_type.add(name="EvaluationKey")
    ek.field.add(name="gk", number=2, type=F.TYPE_MESSAGE, type_name=".pin.GaloisKey", label=F.LABEL_REPEATED)
    ek.field.add(name="ciphertext_level", number=3, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    ek.field.add(name="evaluation_key_level", number=4, type=F.TYPE_UINT32, label=F.LABEL_OPTIONAL)
    pool = descriptor_pool.DescriptorPool()
    pool.Add(fd)
    get = message_factory.GetMessageClass
    return (get(pool.FindMessageTypeByName("pin.Rq")), get(pool.FindMessageTypeByName("pin.Ciphertext")),
            get(pool.FindMessageTypeByName("pin.KeySwitchingKey")), get(pool.FindMessageTypeByName("pin.GaloisKey")),
            get(pool.FindMessageTypeByName("pin.EvaluationKey")))


def test_protobuf_framing_pinned(ora):
    """The oracle's Rq / Ciphertext encoding equals the protobuf package's for
    the same field values (seeded and unseeded, levels 0 and 1, the variable
    time flag), and its decoder inverts it."""
    Rq, Ct, _, _, _ = _proto_classes()
    rng = np.random.default_rng(41)
    par = ora.BfvParameters(16, 1153, moduli_sizes=[62] * 3)
    sk = ora.SecretKey.random(par, rng)
    for level in (0, 1):
        ctx = par.context_at_level(level)
        pt = ora.Plaintext.encode(rng.integers(0, 1153, 16, dtype=np.uint64), "simd", par, level)
        ct = sk.encrypt(pt, rng)
        for seed in (None, bytes(range(32))):
            if seed:
                ct.c[1] = ora.Poly(ctx, ora.random_from_seed(ctx, seed), ora.NTT)
            for avt in (False, True):
                got = ora.ciphertext_message(ct, seed, avt)
                want = Ct(c=[Rq(representation=2, degree=16, coefficients=ora.rq_payload(p),
                                allow_variable_time=avt).SerializeToString() for p in (ct.c[:1] if seed else ct.c)],
                          seed=seed or b"", level=level).SerializeToString()
                assert got == want, (level, seed is not None, avt)
                back = ora.ciphertext_from_message(par, got)
                assert back.level == level and np.array_equal(back.to_array(), ct.to_array())
    # Multi-byte varints: a degree of 2^14 and payloads over 127 bytes.
    assert ora._varint(16384) == b"\x80\x80\x01" and ora._varint(300) == b"\xac\x02"
    with pytest.raises(ValueError):
        ora.ciphertext_from_message(par, ora._pb_bytes(1, b"\x08\x02", repeated=True))


def test_key_messages_pinned(ora):
    """KeySwitchingKey / GaloisKey encoding (key_switching_key.rs:332-352,
    galois_key.rs:127-134) equals the protobuf package's, seeded and not."""
    Rq, _, Ksk, Gk, Ek = _proto_classes()
    rng = np.random.default_rng(43)
    par = ora.BfvParameters(16, 1153, moduli_sizes=[62] * 3)
    sk = ora.SecretKey.random(par, rng)

    def rq(p):
        return Rq(representation=3, degree=16, coefficients=ora.rq_payload(p), allow_variable_time=True)

    for seed in (None, bytes(range(32))):
        gk = ora.GaloisKey(sk, 3, 1, 0, rng, seed=seed)
        k = gk.ksk
        want = Ksk(c0=[rq(p).SerializeToString() for p in k.c0],
                   c1=[] if seed else [rq(p).SerializeToString() for p in k.c1], seed=seed or b"",
                   ciphertext_level=1, ksk_level=0)
        assert ora.ksk_message(k) == want.SerializeToString()
        assert ora.galois_key_message(gk) == Gk(ksk=want, exponent=3).SerializeToString()
    # A decomposition key (single-modulus context: log_base 31) and an
    # EvaluationKey of two Galois keys (evaluation_key.rs:382-392).
    dk = ora.GaloisKey(sk, 5, 2, 2, rng).ksk
    assert ora.ksk_message(dk) == Ksk(c0=[rq(p).SerializeToString() for p in dk.c0],
                                      c1=[rq(p).SerializeToString() for p in dk.c1], ciphertext_level=2,
                                      ksk_level=2, log_base=31).SerializeToString()
    gks = [ora.GaloisKey(sk, e, 1, 0, rng) for e in (3, 2 * 16 - 1)]
    want = Ek(gk=[Gk.FromString(ora.galois_key_message(g)) for g in gks], ciphertext_level=1, evaluation_key_level=0)
    assert ora.evaluation_key_message(gks, 1, 0) == want.SerializeToString()
