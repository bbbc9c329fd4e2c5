"""GPU NTT parity: batched forward / lazy forward / backward through the C ABI,
bit-exact against the oracle's restatement of ntt/native.rs."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _moduli(ora, n, L):
    out, ub = [], 1 << 62
    while len(out) < L:
        ub = ora.generate_prime(62, 2 * n, ub)
        out.append(ub)
    return out


@pytest.mark.parametrize("logn", [3, 4, 5, 10, 12, 13, 14, 15, 16])
@pytest.mark.parametrize("L,B", [(1, 1), (4, 3)])
def test_ntt_forward_backward_bit_exact(fg, ora, cuda, logn, L, B):
    n = 1 << logn
    moduli = _moduli(ora, n, L)
    rng = np.random.default_rng(logn * 100 + L)
    data = np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli]) for _ in range(B)])
    ctx = fg.Context(moduli, n)
    t = fg.to_device(data)
    fg.ntt_forward(ctx, t)
    got_fwd = fg.to_host(t)
    lazy = fg.to_device(data)
    fg.ntt_forward(ctx, lazy, lazy=True)
    got_lazy = fg.to_host(lazy)
    expect = data.copy()
    for b in range(B):
        for i, m in enumerate(moduli):
            ora.ntt_operator(m, n).forward(expect[b, i])
    assert np.array_equal(got_fwd, expect)
    for i, m in enumerate(moduli):
        assert (got_lazy[:, i] < np.uint64(4 * m)).all()
        assert np.array_equal(got_lazy[:, i] % np.uint64(m), expect[:, i])
    fg.ntt_backward(ctx, t)
    assert np.array_equal(fg.to_host(t), data)


PLANS = [(13, 12, 0), (14, 12, 0), (14, 13, 0), (15, 12, 0), (15, 13, 0), (16, 12, 0), (16, 13, 0),
         (13, 12, 1), (14, 12, 1), (15, 12, 1), (16, 12, 1)]


@pytest.mark.parametrize("logn,bl,cluster", PLANS)
def test_ntt_plans_bit_exact(fg, ora, cuda, logn, bl, cluster):
    """Every two-pass plan (strided pass + blocks of 2^bl), and the single-pass
    cluster form of the 2^12-block plans (2 to 16 CTAs per cluster), gives
    the oracle's output, lazy and reduced, and inverts."""
    n = 1 << logn
    moduli = _moduli(ora, n, 3)
    rng = np.random.default_rng(logn * 7 + bl)
    data = np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli]) for _ in range(3)])
    expect = data.copy()
    for b in range(3):
        for i, m in enumerate(moduli):
            ora.ntt_operator(m, n).forward(expect[b, i])
    ctx = fg.Context(moduli, n)
    default = fg.ntt_plan_get(logn)
    default_cluster = fg.ntt_cluster_get(logn)
    try:
        fg.ntt_plan_set(logn, bl)
        fg.ntt_cluster_set(logn, bool(cluster))
        t = fg.to_device(data)
        fg.ntt_forward(ctx, t)
        assert np.array_equal(fg.to_host(t), expect)
        lazy = fg.to_device(data)
        fg.ntt_forward(ctx, lazy, lazy=True)
        got = fg.to_host(lazy)
        for i, m in enumerate(moduli):
            assert (got[:, i] < np.uint64(4 * m)).all()
            assert np.array_equal(got[:, i] % np.uint64(m), expect[:, i])
        fg.ntt_backward(ctx, t)
        assert np.array_equal(fg.to_host(t), data)
    finally:
        fg.ntt_plan_set(logn, default)
        fg.ntt_cluster_set(logn, default_cluster)


def test_ntt_autotune_installs_a_valid_plan(fg, ora, cuda):
    n = 1 << 14
    ctx = fg.Context(_moduli(ora, n, 2), n)
    default = fg.ntt_plan_get(14)
    default_cluster = fg.ntt_cluster_get(14)
    try:
        bl = fg.ntt_autotune(ctx, 8)
        assert bl in (12, 13, 14) and fg.ntt_plan_get(14) == bl
        assert bl == 12 or not fg.ntt_cluster_get(14)
    finally:
        fg.ntt_plan_set(14, default)
        fg.ntt_cluster_set(14, default_cluster)


def test_ntt_lazy_inputs(fg, ora, cuda):
    """Forward NTT accepts lazy [0, 4p) inputs like `forward_vt_lazy`."""
    n, p = 1 << 14, 4611686018427322369
    rng = np.random.default_rng(5)
    base = rng.integers(0, p, n, dtype=np.uint64)
    lazy_in = base + np.uint64(p) * rng.integers(0, 4, n, dtype=np.uint64)
    ctx = fg.Context([p], n)
    t = fg.to_device(lazy_in[None, None])
    fg.ntt_forward(ctx, t)
    expect = base.copy()
    ora.ntt_operator(p, n).forward(expect)
    assert np.array_equal(fg.to_host(t)[0, 0], expect)


def test_ntt_injected_root(fg, ora, cuda):
    """A caller-supplied root (another primitive 2N-th root) is honoured."""
    n, p = 4096, 4611686018427322369
    op = ora.NttOperator(ora.Modulus(p), n)
    root = pow(op.omega, 5, p)
    other = ora.NttOperator(ora.Modulus(p), n, root=root)
    ctx = fg.Context([p], n, roots=[root])
    rng = np.random.default_rng(9)
    a = rng.integers(0, p, n, dtype=np.uint64)
    t = fg.to_device(a[None, None])
    fg.ntt_forward(ctx, t)
    e = a.copy()
    other.forward(e)
    assert np.array_equal(fg.to_host(t)[0, 0], e)


def test_ntt_edge_values(fg, ora, cuda):
    """All-zero and all-(p-1) limbs."""
    n = 1 << 14
    moduli = _moduli(ora, n, 2)
    data = np.stack([np.zeros(n, dtype=np.uint64), np.full(n, moduli[1] - 1, dtype=np.uint64)])[None]
    ctx = fg.Context(moduli, n)
    t = fg.to_device(data)
    fg.ntt_forward(ctx, t)
    expect = data.copy()
    for i, m in enumerate(moduli):
        ora.ntt_operator(m, n).forward(expect[0, i])
    assert np.array_equal(fg.to_host(t), expect)
    fg.ntt_backward(ctx, t)
    assert np.array_equal(fg.to_host(t), data)
