"""Parity on the benchmark configurations themselves, at their full sizes.

Each test names the configuration it covers:
  config 1  ct x ct + relinearization, batch 1, N = 4096, two 62-bit moduli,
            t = 65537, with a ternary secret (the default CBD secret is
            covered by test_gpu_bfv.test_multiply_default);
  config 2  batched negacyclic NTT, N = 2^13 .. 2^16, L = 8 and 16, up to
            256 polynomials per launch;
  config 3  64 ciphertext pairs at N = 2^14, L = 6 through the captured
            two-branch graph, every product against the oracle and against
            64 single-pair launches;
  config 4  32 rotations at N = 2^15 with 4 to 12 live moduli, one key per
            (step, level), in one ragged batch;
  config 5  one server receiving a shuffled mix over all three parameter sets
            (2^13 / L3, 2^14 / L6, 2^15 / L12) at several levels each.
Every GPU output is compared bit for bit with the oracle."""

import numpy as np
import pytest

from test_gpu_bfv import Setup
from test_gpu_serve import _submit

pytestmark = pytest.mark.gpu


def _moduli(ora, n, L):
    out, ub = [], 1 << 62
    while len(out) < L:
        ub = ora.generate_prime(62, 2 * n, ub)
        out.append(ub)
    return out


# ---------------------------------------------------------------------------
# config 1


def test_config1_ternary_secret_mul_relin(fg, ora, cuda):
    rng = np.random.default_rng(101)
    par_o = ora.BfvParameters(4096, 65537, moduli_sizes=[62, 62])
    sk = ora.SecretKey.ternary(par_o, rng)
    assert set(np.unique(sk.coeffs)) <= {-1, 0, 1}
    rk_o = ora.RelinearizationKey(sk, rng)
    par = fg.BfvParameters(4096, par_o.moduli, 65537)
    rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array())
    mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    vals = [rng.integers(0, 65537, 4096, dtype=np.uint64) for _ in range(2)]
    cts = [sk.encrypt(ora.Plaintext.encode(v, "simd", par_o), rng) for v in vals]
    out = fg.to_host(mult.multiply(fg.to_device(cts[0].to_array()[None]), fg.to_device(cts[1].to_array()[None])))[0]
    want = mult_o.multiply(cts[0], cts[1])
    assert np.array_equal(out, want.to_array())
    got = sk.decrypt(ora.Ciphertext.from_array(par_o, out, 0)).decode("simd")
    assert [int(x) for x in got] == [int(a) * int(b) % 65537 for a, b in zip(vals[0], vals[1])]


# ---------------------------------------------------------------------------
# config 2


@pytest.mark.parametrize("logn", [13, 14, 15, 16])
@pytest.mark.parametrize("L", [8, 16])
def test_config2_ntt_every_limb(fg, ora, cuda, logn, L):
    """Forward (reduced and lazy) and inverse of 3 polynomials, every limb
    against the oracle."""
    n = 1 << logn
    moduli = _moduli(ora, n, L)
    rng = np.random.default_rng(logn * 31 + L)
    data = np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli]) for _ in range(3)])
    ctx = fg.Context(moduli, n)
    expect = data.copy()
    for b in range(3):
        for i, m in enumerate(moduli):
            ora.ntt_operator(m, n).forward(expect[b, i])
    t = fg.to_device(data)
    fg.ntt_forward(ctx, t)
    assert np.array_equal(fg.to_host(t), expect)
    lazy = fg.to_device(data)
    fg.ntt_forward(ctx, lazy, lazy=True)
    got = fg.to_host(lazy)
    q = np.array(moduli, dtype=np.uint64)[None, :, None]
    assert (got < 4 * q).all()
    assert np.array_equal(got % q, expect)
    fg.ntt_backward(ctx, t)
    assert np.array_equal(fg.to_host(t), data)


def test_config2_ntt_256_polys_n65536_l16(fg, ora, cuda):
    """The largest launch of the configuration: 256 polynomials of 16 limbs at
    N = 2^16 (2.1 GB). Two whole polynomials and 40 sampled limbs are compared
    with the oracle, reduced and lazy; the inverse restores every limb."""
    torch = cuda
    n, L, B = 1 << 16, 16, 256
    moduli = _moduli(ora, n, L)
    ctx = fg.Context(moduli, n)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(2016)
    q = torch.tensor([int(m) for m in moduli], dtype=torch.int64, device="cuda").view(1, L, 1)
    data = torch.randint(0, 1 << 62, (B, L, n), dtype=torch.int64, device="cuda", generator=gen) % q
    t = data.clone()
    fg.ntt_forward(ctx, t)
    rng = np.random.default_rng(7)
    sampled = [(0, l) for l in range(L)] + [(B - 1, l) for l in range(L)]
    sampled += [(int(b), int(l)) for b, l in zip(rng.integers(1, B - 1, 40), rng.integers(0, L, 40))]
    for b, l in sampled:
        row = fg.to_host(data[b, l])
        ora.ntt_operator(moduli[l], n).forward(row)
        assert np.array_equal(fg.to_host(t[b, l]), row), (b, l)
    lazy = data.clone()
    fg.ntt_forward(ctx, lazy, lazy=True)
    for b, l in sampled[::3]:
        got = fg.to_host(lazy[b, l])
        assert (got < np.uint64(4 * moduli[l])).all()
        assert np.array_equal(got % np.uint64(moduli[l]), fg.to_host(t[b, l])), (b, l)
    del lazy
    fg.ntt_backward(ctx, t)
    assert torch.equal(t, data)


# ---------------------------------------------------------------------------
# config 3


def test_config3_graph_64_pairs_every_product(fg, ora, cuda):
    """The headline workload: 64 pairs at N = 2^14, L = 6 (seven extension
    moduli) replayed as the captured graph of two concurrent 32-pair branches.
    All 64 products equal the oracle's and 64 one-pair launches; four
    decrypt to the slotwise product."""
    s = Setup(fg, ora, 16384, 6, 65537, seed=3064)
    rk_o, rk = s.rk()
    mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
    vals, cts = s.encrypt(64)
    pair = [(i, (7 * i + 3) % 64) for i in range(64)]
    lhs_h = np.stack([cts[i].to_array() for i, _ in pair])
    rhs_h = np.stack([cts[j].to_array() for _, j in pair])
    lhs, rhs = fg.to_device(lhs_h), fg.to_device(rhs_h)
    out = fg.empty((64, 2, 6, 16384))
    g = mult.capture(lhs, rhs, out)
    out.zero_()
    g.launch()
    cuda.cuda.synchronize()
    got = fg.to_host(out)
    for k, (i, j) in enumerate(pair):
        assert np.array_equal(got[k], mult_o.multiply(cts[i], cts[j]).to_array()), f"product {k}"
    for k in range(64):
        single = fg.to_host(mult.multiply(lhs[k:k + 1], rhs[k:k + 1]))[0]
        assert np.array_equal(single, got[k]), f"single launch {k}"
    for k in (0, 21, 42, 63):
        i, j = pair[k]
        assert list(s.decrypt(got[k], 0)) == s.product(vals[i], vals[j])


# ---------------------------------------------------------------------------
# config 4


def test_config4_ragged_rotations_n32768_l12(fg, ora, cuda):
    """32 ciphertexts at N = 2^15, each switched to a random level with 4 to
    12 live moduli and rotated by a step uniform in [1, N/2) with its own
    Galois key (exponent 3^step mod 2N), in one ragged batch (two
    concurrent halves of 16)."""
    n, top = 32768, 12
    s = Setup(fg, ora, n, top, 65537, seed=4032)
    rng = np.random.default_rng(4)
    live = [int(x) for x in rng.integers(4, top + 1, 32)]
    steps = [int(x) for x in rng.integers(1, n // 2, 32)]
    keys, cts_d, want, vals = [], [], [], []
    for b in range(32):
        lvl = top - live[b]
        e = ora.rotation_exponent(s.par_o, steps[b])
        gk_o = ora.GaloisKey(s.sk, e, lvl, lvl, s.rng)
        keys.append(fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), lvl, lvl))
        v, cts = s.encrypt(1, level=lvl)
        vals.append(v[0])
        cts_d.append(fg.to_device(cts[0].to_array()))
        want.append(gk_o.relinearize(cts[0]).to_array())
        del gk_o
    assert min(live) <= 5 and max(live) >= 11  # the draw spans the range
    outs = fg.rotate_batch(s.par, keys, cts_d)
    half = n // 2
    for b in range(32):
        got = fg.to_host(outs[b])
        assert np.array_equal(got, want[b]), f"entry {b} ({live[b]} moduli, step {steps[b]})"
    for b in (0, 31):
        v, i = vals[b], steps[b]
        rot = np.concatenate([np.roll(v[:half], -i), np.roll(v[half:], -i)])
        assert np.array_equal(s.decrypt(fg.to_host(outs[b]), top - live[b]), rot)


# ---------------------------------------------------------------------------
# config 5


def _config5_requests(fg, ora, s, levels, per_kind, keep):
    """mul+relin, rotations, additions and switch-downs of one parameter set
    at `levels`, with the oracle's results."""
    reqs = []
    for lvl in levels:
        rk_o, rk = s.rk(lvl)
        mult_o, mult = ora.Multiplicator.default(rk_o), fg.Multiplicator.default(rk)
        keep.append(mult)
        e = ora.rotation_exponent(s.par_o, 1 + lvl) if lvl % 2 else 2 * s.n - 1
        gk_o = ora.GaloisKey(s.sk, e, lvl, lvl, s.rng)
        gk = fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), lvl, lvl)
        keep.append(gk)
        _, cts = s.encrypt(5 * per_kind, level=lvl)
        for i in range(per_kind):
            a, b, c, d, f = cts[5 * i:5 * i + 5]
            reqs.append(("mul", (mult, a.to_array(), b.to_array()), mult_o.multiply(a, b).to_array()))
            reqs.append(("rot", (gk, c.to_array()), gk_o.relinearize(c).to_array()))
            reqs.append(("add", (s.par, lvl, d.to_array(), f.to_array()), (d + f).to_array()))
            if lvl < s.par_o.max_level():
                reqs.append(("down", (s.par, lvl, f.to_array()), f.copy().switch_down().to_array()))
    return reqs


def test_config5_server_mix_over_three_parameter_sets(fg, ora, cuda):
    """One server receives, shuffled, requests of every kind over N = 2^13
    (L = 3), 2^14 (L = 6) and 2^15 (L = 12) at two levels each: every result
    equals the same request alone and the oracle."""
    keep, reqs = [], []
    for (n, L, levels) in [(8192, 3, (0, 1)), (16384, 6, (0, 3)), (32768, 12, (0, 7))]:
        s = Setup(fg, ora, n, L, 65537, seed=5000 + n)
        keep.append(s)
        reqs += _config5_requests(fg, ora, s, levels, 2, keep)
    order = np.random.default_rng(5).permutation(len(reqs))
    with fg.Server(hbm_budget_bytes=8 << 30, streams=4, max_batch=16) as srv:
        ids = {idx: _submit(srv, *reqs[idx][:2]) for idx in order}
        mixed = {idx: srv.wait(rid) for idx, rid in ids.items()}
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["batches"] < len(reqs)
        for idx, (kind, args, want) in enumerate(reqs):
            assert np.array_equal(mixed[idx], want), f"request {idx} ({kind}) in the mix vs oracle"
            alone = srv.wait(_submit(srv, kind, args))
            assert np.array_equal(alone, want), f"request {idx} ({kind}) alone vs oracle"
