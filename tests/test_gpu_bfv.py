"""GPU BFV hot path (crate fhe) bit-exact against the oracle and decrypting
correctly: Multiplicator (mul+relin, mod switching, no relinearization, custom
strategy, levels), relinearization, rotations, switch-down and addition."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Setup:
    def __init__(self, fg, ora, n, L, t, seed, level=0):
        self.rng = np.random.default_rng(seed)
        self.ora, self.fg, self.n, self.t, self.level = ora, fg, n, t, level
        self.par_o = ora.BfvParameters(n, t, moduli_sizes=[62] * L)
        self.sk = ora.SecretKey.random(self.par_o, self.rng)
        self.par = fg.BfvParameters(n, self.par_o.moduli, t)

    def encrypt(self, count, level=None):
        level = self.level if level is None else level
        vals, cts = [], []
        for _ in range(count):
            v = self.rng.integers(0, self.t, self.n, dtype=np.uint64)
            vals.append(v)
            cts.append(self.sk.encrypt(self.ora.Plaintext.encode(v, "simd", self.par_o, level), self.rng))
        return vals, cts

    def rk(self, level=None):
        level = self.level if level is None else level
        rk_o = self.ora.RelinearizationKey(self.sk, self.rng, level, level)
        rk = self.fg.RelinearizationKey(self.par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), level, level)
        return rk_o, rk

    def decrypt(self, arr, level):
        return self.sk.decrypt(self.ora.Ciphertext.from_array(self.par_o, arr, level)).decode("simd")

    def product(self, a, b):
        return [int(x) * int(y) % self.t for x, y in zip(a, b)]


@pytest.mark.parametrize("n,L,t,B", [(16, 3, 1153, 3), (4096, 2, 65537, 2), (16384, 6, 65537, 2),
                                     (32768, 3, 65537, 1), (32768, 12, 65537, 2), (8192, 3, 65537, 2)])
def test_multiply_default(fg, ora, cuda, n, L, t, B):
    s = Setup(fg, ora, n, L, t, seed=n + L)
    rk_o, rk = s.rk()
    mult_o = ora.Multiplicator.default(rk_o)
    mult = fg.Multiplicator.default(rk)
    vals, cts = s.encrypt(2 * B)
    lhs = np.stack([c.to_array() for c in cts[:B]])
    rhs = np.stack([c.to_array() for c in cts[B:]])
    out = fg.to_host(mult.multiply(fg.to_device(lhs), fg.to_device(rhs)))
    assert out.shape == (B, 2, L, n)
    for b in range(B):
        want = mult_o.multiply(cts[b], cts[B + b]).to_array()
        assert np.array_equal(out[b], want), f"pair {b}"
        assert list(s.decrypt(out[b], 0)) == s.product(vals[b], vals[B + b])


@pytest.mark.parametrize("n,L,B", [(8192, 3, 3), (16384, 6, 33), (32768, 12, 2)])
def test_multiply_tensor_core_scalers(fg, ora, cuda, n, L, B):
    """The multiplication with its scalers of 12 or more source moduli on the
    tensor cores (the default: the L = 6 scale-down, the L = 12 extension)
    equals the same multiplication on the CUDA cores, for every pair, and the
    oracle's product for the first and last (33 pairs run as two concurrent
    halves; L = 3 has no such scaler and checks the switch alone)."""
    s = Setup(fg, ora, n, L, 65537, seed=n + 7 * L)
    rk_o, rk = s.rk()
    mult = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(4)
    lhs = fg.to_device(np.stack([cts[b % 2].to_array() for b in range(B)]))
    rhs = fg.to_device(np.stack([cts[2 + b % 2].to_array() for b in range(B)]))
    default = fg.rns_tensor_get()
    try:
        fg.rns_tensor_set(True)
        on = fg.to_host(mult.multiply(lhs, rhs))
        fg.rns_tensor_set(False)
        off = fg.to_host(mult.multiply(lhs, rhs))
    finally:
        fg.rns_tensor_set(default)
    assert fg.rns_tensor_wait_failures() == 0
    assert np.array_equal(on, off)
    mult_o = ora.Multiplicator.default(rk_o)
    for b in (0, B - 1):
        assert np.array_equal(on[b], mult_o.multiply(cts[b % 2], cts[2 + b % 2]).to_array()), b


def test_multiply_variants(fg, ora, cuda):
    """mul.rs:246-339: mod switching and no relinearization."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=77)
    rk_o, rk = s.rk()
    vals, cts = s.encrypt(2)
    lhs, rhs = (fg.to_device(c.to_array()[None]) for c in cts)
    want_vals = s.product(vals[0], vals[1])
    # mod switching
    mo = ora.Multiplicator.default(rk_o)
    mo.enable_mod_switching()
    m = fg.Multiplicator.default(rk)
    m.enable_mod_switching()
    assert m.output_shape() == (2, 1)
    out = fg.to_host(m.multiply(lhs, rhs))[0]
    want = mo.multiply(cts[0], cts[1])
    assert want.level == 1 and np.array_equal(out, want.to_array())
    assert list(s.decrypt(out, 1)) == want_vals
    # no relinearization (3 parts), via a leveled multiplicator with the default basis
    ext = ora.Multiplicator.default_extended_basis(s.par_o, 0)
    q = s.par_o.context_at_level(0).modulus()
    mo3 = ora.Multiplicator(ora.ScalingFactor.one(), ora.ScalingFactor.one(), ext,
                            ora.ScalingFactor(65537, q), 0, s.par_o)
    m3 = fg.Multiplicator.new_leveled(fg.ScalingFactor.one(), fg.ScalingFactor.one(), ext,
                                      fg.ScalingFactor(65537, q), 0, s.par)
    assert m3.output_shape() == (3, 0)
    out3 = fg.to_host(m3.multiply(lhs, rhs))[0]
    want3 = mo3.multiply(cts[0], cts[1])
    assert np.array_equal(out3, want3.to_array())
    assert list(s.decrypt(out3, 0)) == want_vals
    # relinearize the 3-part product separately (relinearization_key.rs:71-98)
    out_r = fg.to_host(rk.relinearizes(fg.to_device(out3[None])))[0]
    assert np.array_equal(out_r, rk_o.relinearizes(want3).to_array())
    assert list(s.decrypt(out_r, 0)) == want_vals


def test_multiply_custom_strategy(fg, ora, cuda):
    """mul.rs:341-401: the second strategy of eprint 2021/204 (rhs scaled by P/Q)."""
    s = Setup(fg, ora, 16, 3, 1153, seed=5)
    ext = list(s.par_o.moduli)
    for k in range(3):
        ext.append(ora.generate_prime(62, 2 * 16, ext[2 + k]))
    rns = ora.RnsContext(ext[3:])
    q = s.par_o.context_at_level(0).modulus()
    args_o = (ora.ScalingFactor.one(), ora.ScalingFactor(rns.modulus(), q), ext,
              ora.ScalingFactor(1153, rns.modulus()), 0, s.par_o)
    mo = ora.Multiplicator(*args_o)
    m = fg.Multiplicator.new_leveled(fg.ScalingFactor.one(), fg.ScalingFactor(rns.modulus(), q), ext,
                                     fg.ScalingFactor(1153, rns.modulus()), 0, s.par)
    vals, cts = s.encrypt(2)
    out = fg.to_host(m.multiply(fg.to_device(cts[0].to_array()[None]), fg.to_device(cts[1].to_array()[None])))[0]
    want = mo.multiply(cts[0], cts[1])
    assert np.array_equal(out, want.to_array())
    assert list(s.decrypt(out, 0)) == s.product(vals[0], vals[1])


def test_multiply_at_level(fg, ora, cuda):
    """mul.rs:281-317: keys and ciphertexts at level 1."""
    s = Setup(fg, ora, 4096, 3, 65537, seed=9, level=1)
    rk_o, rk = s.rk()
    vals, cts = s.encrypt(2)
    assert cts[0].level == 1
    mo, m = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    out = fg.to_host(m.multiply(fg.to_device(cts[0].to_array()[None]), fg.to_device(cts[1].to_array()[None])))[0]
    assert np.array_equal(out, mo.multiply(cts[0], cts[1]).to_array())
    assert list(s.decrypt(out, 1)) == s.product(vals[0], vals[1])


def test_graph_replay(fg, ora, cuda):
    """A captured multiplication replays the pipeline on whatever the input
    buffers hold at launch time, bit-exact with multiply()."""
    s = Setup(fg, ora, 16384, 3, 65537, seed=31)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(8)
    first = [np.stack([c.to_array() for c in cts[k:k + 2]]) for k in (0, 2)]
    second = [np.stack([c.to_array() for c in cts[k:k + 2]]) for k in (4, 6)]
    lhs, rhs = fg.to_device(first[0]), fg.to_device(first[1])
    out = fg.empty((2, 2, 3, 16384))
    g = m.capture(lhs, rhs, out)
    assert g.kernels >= 7
    want1 = fg.to_host(m.multiply(lhs, rhs))
    assert np.array_equal(fg.to_host(out), want1)
    lhs.copy_(fg.to_device(second[0]))
    rhs.copy_(fg.to_device(second[1]))
    g.launch()
    cuda.cuda.synchronize()
    want2 = fg.to_host(m.multiply(lhs, rhs))
    assert np.array_equal(fg.to_host(out), want2)
    mo = ora.Multiplicator.default(rk_o)
    assert np.array_equal(want2[1], mo.multiply(cts[5], cts[7]).to_array())


@pytest.mark.parametrize("count", [32, 33])
def test_graph_two_branches(fg, ora, cuda, count):
    """Batches of 32 pairs or more run as two concurrent halves, each with its
    own scratch (33 splits 16 + 17), both as direct calls and as captured
    graphs. Every product of both forms equals the single-pass path (chunks of
    fewer than 32 pairs), and two products equal the oracle's."""
    s = Setup(fg, ora, 4096, 2, 65537, seed=41 + count)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    q = np.array(s.par_o.moduli, dtype=np.uint64)[None, None, :, None]
    rng = np.random.default_rng(count)
    lhs_h = (rng.integers(0, 1 << 62, (count, 2, 2, 4096), dtype=np.uint64) % q).astype(np.uint64)
    rhs_h = (rng.integers(0, 1 << 62, (count, 2, 2, 4096), dtype=np.uint64) % q).astype(np.uint64)
    lhs, rhs = fg.to_device(lhs_h), fg.to_device(rhs_h)
    single_pass = np.concatenate([
        fg.to_host(m.multiply(fg.to_device(lhs_h[k:k + 12]), fg.to_device(rhs_h[k:k + 12])))
        for k in range(0, count, 12)])
    out = fg.empty((count, 2, 2, 4096))
    g = m.capture(lhs, rhs, out)
    assert g.kernels >= 14
    want = fg.to_host(m.multiply(lhs, rhs))
    assert np.array_equal(want, single_pass)
    out.zero_()
    g.launch()
    cuda.cuda.synchronize()
    assert np.array_equal(fg.to_host(out), single_pass)
    mo = ora.Multiplicator.default(rk_o)
    for b in (0, count - 1):
        lo = ora.Ciphertext.from_array(s.par_o, lhs_h[b], 0)
        ro = ora.Ciphertext.from_array(s.par_o, rhs_h[b], 0)
        assert np.array_equal(want[b], mo.multiply(lo, ro).to_array()), b


def test_batched_equals_single_and_host(fg, ora, cuda):
    """A batch of 6 equals 6 single launches and the host entry point."""
    s = Setup(fg, ora, 4096, 2, 65537, seed=21)
    _, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(12)
    lhs = np.stack([c.to_array() for c in cts[:6]])
    rhs = np.stack([c.to_array() for c in cts[6:]])
    batched = fg.to_host(m.multiply(fg.to_device(lhs), fg.to_device(rhs)))
    for b in range(6):
        single = fg.to_host(m.multiply(fg.to_device(lhs[b:b + 1]), fg.to_device(rhs[b:b + 1])))
        assert np.array_equal(single[0], batched[b])
    assert np.array_equal(m.multiply_host(lhs, rhs), batched)
    # Every pipeline shape (ragged last chunks, 1 to 4 streams) gives the same product.
    for chunk, streams in [(1, 1), (2, 4), (4, 3), (5, 2), (0, 3)]:
        m.set_host_pipeline(chunk, streams)
        assert np.array_equal(m.multiply_host(lhs, rhs), batched), (chunk, streams)
    for bad in (0, 5):
        with pytest.raises(fg.FhegError):
            m.set_host_pipeline(2, bad)


@pytest.mark.parametrize("n,L", [(16, 3), (4096, 2), (32768, 4)])
def test_rotations(fg, ora, cuda, n, L):
    """evaluation_key.rs:92-131 via GaloisKey::relinearize_into."""
    s = Setup(fg, ora, n, L, 65537 if n > 16 else 1153, seed=n * 3 + L)
    steps = [1, 5] if n > 16 else [1, 3]
    ek_o = ora.EvaluationKey(s.sk, s.rng, columns=steps, row_rotation=True)
    gks = [fg.GaloisKey(s.par, e, g.ksk.c0_array(), g.ksk.c1_array()) for e, g in ek_o.gk.items()]
    ek = fg.EvaluationKey(s.par, gks)
    vals, cts = s.encrypt(2)
    batch = fg.to_device(np.stack([c.to_array() for c in cts]))
    half = n // 2
    for i in steps:
        got = fg.to_host(ek.rotates_columns_by(batch, i))
        for b in range(2):
            assert np.array_equal(got[b], ek_o.rotates_columns_by(cts[b], i).to_array())
            want = np.concatenate([np.roll(vals[b][:half], -i), np.roll(vals[b][half:], -i)])
            assert np.array_equal(s.decrypt(got[b], 0), want)
    got = fg.to_host(ek.rotates_rows(batch))
    for b in range(2):
        assert np.array_equal(got[b], ek_o.rotates_rows(cts[b]).to_array())


def test_ciphertext_switch_down_and_add(fg, ora, cuda):
    s = Setup(fg, ora, 4096, 3, 65537, seed=31)
    vals, cts = s.encrypt(2)
    a = np.stack([c.to_array() for c in cts])
    got = fg.to_host(fg.ciphertext_switch_down(s.par, 0, fg.to_device(a)))
    for b in range(2):
        want = cts[b].copy().switch_down()
        assert np.array_equal(got[b], want.to_array())
        assert np.array_equal(s.decrypt(got[b], 1), vals[b])
    ssum = fg.to_host(fg.ciphertext_add(s.par, 0, fg.to_device(a[:1]), fg.to_device(a[1:])))[0]
    assert np.array_equal(ssum, (cts[0] + cts[1]).to_array())
    assert list(s.decrypt(ssum, 0)) == [(int(x) + int(y)) % 65537 for x, y in zip(vals[0], vals[1])]


def test_errors(fg, ora, cuda):
    """Reference error behaviour at the boundary (mul.rs:146-173,
    key_switching_key.rs:219-223, relinearization_key.rs:52-56,
    rq/mod.rs:99-105)."""
    s = Setup(fg, ora, 16, 3, 1153, seed=41)
    _, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    x2 = fg.to_device(np.zeros((1, 2, 3, 16), dtype=np.uint64))
    x3 = fg.to_device(np.zeros((1, 3, 3, 16), dtype=np.uint64))
    with pytest.raises(fg.FhegError):  # wrong number of parts
        m.multiply(x2, x3)
    q = s.par_o.context_at_level(2).modulus()
    ext = ora.Multiplicator.default_extended_basis(s.par_o, 2)
    last = fg.Multiplicator.new_leveled(fg.ScalingFactor.one(), fg.ScalingFactor.one(), ext,
                                        fg.ScalingFactor(1153, q), 2, s.par)
    with pytest.raises(fg.FhegError) as e:  # already the last level
        last.enable_mod_switching()
    assert e.value.code == fg.ERR_NO_MORE_CONTEXT
    with pytest.raises(fg.FhegError) as e:  # even exponent
        fg.substitute(s.par.context_at_level(0), x2[0], 2, 1)
    assert e.value.code == fg.ERR_INVALID_ARGUMENT
    c = np.zeros((2, 3, 16), dtype=np.uint64)
    with pytest.raises(fg.FhegError) as e:  # digit count != ciphertext moduli
        fg.RelinearizationKey(s.par, c, c)
    assert e.value.code == fg.ERR_KEY_MISMATCH
    one = np.zeros((1, 1, 16), dtype=np.uint64)
    with pytest.raises(fg.FhegError) as e:  # single-modulus key context: two base-2^31 digits, not one
        fg.RelinearizationKey(s.par, one, one, 2, 2)
    assert e.value.code == fg.ERR_KEY_MISMATCH
    with pytest.raises(fg.FhegError) as e:
        s.par.context_at_level(3)
    assert e.value.code == fg.ERR_INVALID_LEVEL


@pytest.mark.parametrize("n,L,count", [(4096, 4, 6), (32768, 5, 4), (4096, 4, 17)])
def test_rotate_ragged_batch(fg, ora, cuda, n, L, count):
    """Ciphertexts at different levels, each rotated with its own key in one
    batched call, equal the oracle's one-at-a-time GaloisKey::relinearize
    (17 requests run as two concurrent halves of 8 and 9)."""
    s = Setup(fg, ora, n, L, 65537, seed=1000 + n + L)
    rng = np.random.default_rng(77)
    levels = [int(x) for x in rng.integers(0, L - 1, count)]  # keep >= 2 moduli
    steps = [int(x) for x in rng.integers(1, n // 2, count)]
    keys, cts_o, cts_d, want = [], [], [], []
    for b in range(count):
        lvl = levels[b]
        e = ora.rotation_exponent(s.par_o, steps[b]) if b % 3 else 2 * n - 1
        gk_o = ora.GaloisKey(s.sk, e, lvl, lvl, s.rng)
        keys.append(fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), lvl, lvl))
        _, cts = s.encrypt(1, level=lvl)
        cts_o.append(cts[0])
        cts_d.append(fg.to_device(cts[0].to_array()))
        want.append(gk_o.relinearize(cts[0]).to_array())
    outs = fg.rotate_batch(s.par, keys, cts_d)
    for b in range(count):
        assert np.array_equal(fg.to_host(outs[b]), want[b]), f"entry {b} (level {levels[b]})"


def test_multiply_groups_mixed_levels(fg, ora, cuda):
    """A batch of pairs at four levels, grouped by level (one multiplicator
    per level, one of them with its key two levels below) and issued together:
    every product equals the oracle's and the per-level direct call."""
    n, L = 4096, 5
    s = Setup(fg, ora, n, L, 65537, seed=1400)
    mults, mults_o, lhs, rhs, pairs = [], [], [], [], []
    for lvl, count, klvl in [(0, 5, 0), (1, 3, 1), (2, 4, 0), (3, 2, 3)]:
        rk_o = ora.RelinearizationKey(s.sk, s.rng, lvl, klvl)
        rk = fg.RelinearizationKey(s.par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), lvl, klvl)
        mults.append(fg.Multiplicator.default(rk))
        mults_o.append(ora.Multiplicator.default(rk_o))
        _, cts = s.encrypt(2 * count, level=lvl)
        pairs.append(cts)
        lhs.append(fg.to_device(np.stack([c.to_array() for c in cts[:count]])))
        rhs.append(fg.to_device(np.stack([c.to_array() for c in cts[count:]])))
    outs = fg.multiply_groups(mults, lhs, rhs)
    cuda.cuda.synchronize()
    for g, (m, mo, cts) in enumerate(zip(mults, mults_o, pairs)):
        count = lhs[g].shape[0]
        got = fg.to_host(outs[g])
        assert np.array_equal(got, fg.to_host(m.multiply(lhs[g], rhs[g]))), g
        for b in range(count):
            assert np.array_equal(got[b], mo.multiply(cts[b], cts[count + b]).to_array()), (g, b)
    with pytest.raises(fg.FhegError):
        fg.multiply_groups([mults[0], mults[0]], lhs[:1] * 2, rhs[:1] * 2)


@pytest.mark.parametrize("count", [5, 17])
def test_rotate_batch_graph(fg, ora, cuda, count):
    """A ragged rotation batch (levels 0-2, some keys below the ciphertext
    level; 17 requests as two concurrent halves) recorded as a CUDA graph:
    each replay equals the direct batched call on what the buffers hold."""
    n, L = 4096, 4
    s = Setup(fg, ora, n, L, 65537, seed=1300 + count)
    rng = np.random.default_rng(count)
    keys, want_keys = [], []
    levels = [int(x) for x in rng.integers(0, L - 1, count)]
    for b in range(count):
        lvl = levels[b]
        klvl = lvl if b % 2 else int(rng.integers(0, lvl + 1))
        e = ora.rotation_exponent(s.par_o, int(rng.integers(1, n // 2)))
        gk_o = ora.GaloisKey(s.sk, e, lvl, klvl, s.rng)
        want_keys.append(gk_o)
        keys.append(fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), lvl, klvl))
    cts = [fg.to_device(s.encrypt(1, level=lv)[1][0].to_array()) for lv in levels]
    outs = [fg.empty(c.shape) for c in cts]
    g = fg.capture_rotate_batch(s.par, keys, cts, outs)
    assert g.kernels >= 3
    for rep in range(2):
        fresh = [s.encrypt(1, level=lv)[1][0] for lv in levels]
        for c, f in zip(cts, fresh):
            c.copy_(fg.to_device(f.to_array()))
        for o in outs:
            o.zero_()
        g.launch()
        cuda.cuda.synchronize()
        direct = fg.rotate_batch(s.par, keys, cts)
        for b in range(count):
            got = fg.to_host(outs[b])
            assert np.array_equal(got, fg.to_host(direct[b])), (rep, b)
            assert np.array_equal(got, want_keys[b].relinearize(fresh[b]).to_array()), (rep, b)


@pytest.mark.parametrize("n,plans", [(16384, [12, 13]), (32768, [12, 13])])
def test_pipelines_under_every_ntt_plan(fg, ora, cuda, n, plans):
    """mul+relin, a rotation and a switch-down give the same bytes under every
    NTT plan of their degree (the plan only changes the GPU schedule)."""
    s = Setup(fg, ora, n, 3, 65537, seed=n + 3)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    m.set_small_plan(0)
    gk_o = ora.GaloisKey(s.sk, 2 * n - 1, 0, 0, s.rng)
    gk = fg.GaloisKey(s.par, 2 * n - 1, gk_o.ksk.c0_array(), gk_o.ksk.c1_array())
    _, cts = s.encrypt(2)
    a, b = fg.to_device(cts[0].to_array()[None]), fg.to_device(cts[1].to_array()[None])
    logn = n.bit_length() - 1

    def run():
        return (fg.to_host(m.multiply(a, b)), fg.to_host(gk.relinearize(a)),
                fg.to_host(fg.ciphertext_switch_down(s.par, 0, a.clone())))

    want = (ora.Multiplicator.default(rk_o).multiply(cts[0], cts[1]).to_array(),
            gk_o.relinearize(cts[0]).to_array(), cts[0].copy().switch_down().to_array())
    default = fg.ntt_plan_get(logn)
    default_cluster = fg.ntt_cluster_get(logn)
    try:
        for bl, cluster in [(b, False) for b in plans] + [(12, True), (default, default_cluster)]:
            fg.ntt_plan_set(logn, bl)
            fg.ntt_cluster_set(logn, cluster)
            got = run()
            for g, w in zip(got, want):
                assert np.array_equal(g[0], w), f"plan {bl} cluster {cluster}"
    finally:
        fg.ntt_plan_set(logn, default)
        fg.ntt_cluster_set(logn, default_cluster)


def test_multiplicator_stage_plans_and_times(fg, ora, cuda):
    """Per-stage NTT plans (including the two-launch F stage) leave the product
    unchanged; the autotuner installs a valid plan; stage times are reported."""
    s = Setup(fg, ora, 16384, 3, 65537, seed=404)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    m.set_small_plan(0)  # two pairs would otherwise run with the small-batch plan
    _, cts = s.encrypt(4)
    lhs = fg.to_device(np.stack([cts[0].to_array(), cts[1].to_array()]))
    rhs = fg.to_device(np.stack([cts[2].to_array(), cts[3].to_array()]))
    mo = ora.Multiplicator.default(rk_o)
    want = np.stack([mo.multiply(cts[0], cts[2]).to_array(), mo.multiply(cts[1], cts[3]).to_array()])
    for plan in ([14, 14, 14, 14, 0, 0], [14, 14, 14, 14, 1, 1], [12, 13, 12, 13, 0, 1], [13, 12, 14, 12, 1, 0]):
        m.plan = plan
        assert m.plan == plan
        assert np.array_equal(fg.to_host(m.multiply(lhs, rhs)), want), plan
    with pytest.raises(fg.FhegError):
        m.plan = [15, 14, 14, 14, 0, 0]
    tuned = m.autotune(2)
    assert all(b in (12, 13, 14) for b in tuned[:4]) and len(tuned) == 6 and m.plan == tuned
    out = fg.empty((2, 2, 3, 16384))
    ms = m.stage_times(lhs, rhs, out)
    assert list(ms) == list("ABCDEFG") and all(v > 0 for v in ms.values())
    assert np.array_equal(fg.to_host(out), want)


def test_switch_to_level(fg, ora, cuda):
    """Ciphertext::switch_to_level (ciphertext.rs:100-119) = repeated switch_down."""
    s = Setup(fg, ora, 4096, 5, 65537, seed=91)
    vals, cts = s.encrypt(3)
    arr = np.stack([c.to_array() for c in cts])
    for target in (0, 1, 3, 4):
        got = fg.to_host(fg.ciphertext_switch_to_level(s.par, 0, target, fg.to_device(arr)))
        for b in range(3):
            c = cts[b].copy()
            for _ in range(target):
                c.switch_down()
            assert np.array_equal(got[b], c.to_array()), (target, b)
            assert list(s.decrypt(got[b], target)) == [int(v) for v in vals[b]]
    with pytest.raises(fg.FhegError) as e:
        fg.ciphertext_switch_to_level(s.par, 2, 1, fg.to_device(arr))
    assert e.value.code == fg.ERR_INVALID_LEVEL


def test_errors_of_the_wider_api(fg, ora, cuda):
    """Error statuses of the plaintext side, compositions and wire format."""
    s = Setup(fg, ora, 16, 3, 1153, seed=99)
    _, cts = s.encrypt(2)
    ct = fg.to_device(np.stack([c.to_array() for c in cts]))
    ctx = s.par.context_at_level(0)
    with pytest.raises(fg.FhegError) as e:  # no representation 3
        fg.check(fg.lib().fheg_poly_serialize(ctx._h, 3, None, None, 0, None))
    assert e.value.code == fg.ERR_INVALID_ARGUMENT
    sk = fg.SecretKey(s.par, s.sk.coeffs)
    with pytest.raises(fg.FhegError) as e:
        sk.decrypt(ct[:, :1].contiguous())
    assert e.value.code == fg.ERR_WRONG_PARTS
    with pytest.raises(fg.FhegError) as e:
        fg.dot_product_scalar(s.par, 0, ct[:0], fg.empty((0, 3, 16)))
    assert e.value.code == fg.ERR_INVALID_ARGUMENT
    gk_o = ora.GaloisKey(s.sk, 17, 1, 1, s.rng)
    gk1 = fg.GaloisKey(s.par, 17, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), 1, 1)
    with pytest.raises(fg.FhegError) as e:
        fg.expand(s.par, [gk1], ct[0], 4)  # two levels need two keys
    assert e.value.code == fg.ERR_INVALID_ARGUMENT
    # SIMD needs t = 1 mod 2N
    par2_o = ora.BfvParameters(16, 1031, moduli_sizes=[62] * 2)
    par2 = fg.BfvParameters(16, par2_o.moduli, 1031)
    with pytest.raises(fg.FhegError) as e:
        fg.plaintext_encode(par2, 0, fg.to_device(np.zeros((1, 16), dtype=np.uint64)))
    assert e.value.code == fg.ERR_UNSUPPORTED
    fg.plaintext_encode(par2, 0, fg.to_device(np.zeros((1, 16), dtype=np.uint64)), simd=False)


def test_item_count_bound(fg, ora, cuda):
    """Counts above 2^24 items are refused before any size is derived from
    them (so none can wrap around to a small scratch allocation); the
    buffers passed are far smaller than such a count would need, and no
    kernel runs."""
    s = Setup(fg, ora, 16, 3, 1153, seed=98)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(2)
    ct = fg.to_device(np.stack([c.to_array() for c in cts]))
    out = fg.empty(tuple(ct.shape))
    ctx = s.par.context_at_level(0)
    huge = (1 << 24) + 1
    dp, st = fg._dp, fg._stream()
    calls = [
        lambda: fg.lib().fheg_ntt_forward(ctx._h, dp(ct), huge, 0, st),
        lambda: fg.lib().fheg_poly_op(ctx._h, 0, dp(ct), dp(ct), dp(out), huge, st),
        lambda: fg.lib().fheg_multiplicator_multiply(m._h, dp(ct), dp(ct), dp(out), huge, st),
        lambda: fg.lib().fheg_relinearize(rk._h, dp(ct), dp(out), huge, st),
        lambda: fg.lib().fheg_ciphertext_add(s.par._h, 0, 2, dp(ct), dp(ct), dp(out), huge, st),
    ]
    for call in calls:
        with pytest.raises(fg.FhegError) as e:
            fg.check(call())
        assert e.value.code == fg.ERR_INVALID_ARGUMENT and "2^24" in str(e.value)
    cuda.cuda.synchronize()
    assert np.array_equal(fg.to_host(ct), np.stack([c.to_array() for c in cts]))


def test_small_batch_plan(fg, ora, cuda):
    """Batches up to the small-batch threshold use their own plan; results
    are the same with it, without it and with a custom one."""
    s = Setup(fg, ora, 16384, 3, 65537, seed=405)
    rk_o, rk = s.rk()
    m = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(2)
    a, b = fg.to_device(cts[0].to_array()[None]), fg.to_device(cts[1].to_array()[None])
    want = ora.Multiplicator.default(rk_o).multiply(cts[0], cts[1]).to_array()
    assert np.array_equal(fg.to_host(m.multiply(a, b))[0], want)  # default small plan
    m.set_small_plan(0)
    assert np.array_equal(fg.to_host(m.multiply(a, b))[0], want)
    m.set_small_plan(4, [13, 12, 13, 12, 0, 1])
    assert np.array_equal(fg.to_host(m.multiply(a, b))[0], want)
    with pytest.raises(fg.FhegError):
        m.set_small_plan(4, [11, 12, 12, 12, 0, 0])
    big = m.plan
    tuned = m.autotune(2)  # within the threshold: tunes the small-batch plan only
    assert m.plan == big and all(b in (12, 13, 14) for b in tuned[:4])
    assert np.array_equal(fg.to_host(m.multiply(a, b))[0], want)
