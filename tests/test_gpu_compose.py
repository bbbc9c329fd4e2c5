"""Compositions of the key-switching path against the oracle: inner sum and
oblivious expansion (EvaluationKey), and the ciphertext-plaintext dot product."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


def _gk(fg, ora, s, exps, level=0):
    keys_o, keys = [], []
    for e in exps:
        g = ora.GaloisKey(s.sk, e, level, level, s.rng)
        keys_o.append(g)
        keys.append(fg.GaloisKey(s.par, e, g.ksk.c0_array(), g.ksk.c1_array(), level, level))
    return keys_o, keys


@pytest.mark.parametrize("n,L,t,level", [(16, 3, 1153, 0), (4096, 3, 65537, 1), (16384, 4, 65537, 0)])
def test_inner_sum(fg, ora, cuda, n, L, t, level):
    s = Setup(fg, ora, n, L, t, seed=n + 17)
    exps = ora.EvaluationKey.inner_sum_exponents(s.par_o)
    keys_o, keys = _gk(fg, ora, s, exps, level)
    ek = ora.EvaluationKey(s.sk, s.rng, ciphertext_level=level, evaluation_key_level=level)
    ek.gk = dict(zip(exps, keys_o))
    vals, cts = s.encrypt(2, level=level)
    got = fg.to_host(fg.inner_sum(s.par, keys, fg.to_device(np.stack([c.to_array() for c in cts]))))
    for b in range(2):
        want = ek.computes_inner_sum(cts[b])
        assert np.array_equal(got[b], want.to_array())
        assert set(int(x) for x in s.decrypt(got[b], level)) == {int(np.asarray(vals[b], dtype=object).sum()) % t}


@pytest.mark.parametrize("n,L,size", [(16, 3, 5), (4096, 2, 8), (16384, 3, 3)])
def test_expand(fg, ora, cuda, n, L, size):
    s = Setup(fg, ora, n, L, 65537 if n > 16 else 1153, seed=n + size)
    level = max(size - 1, 0).bit_length()
    exps = ora.EvaluationKey.expansion_exponents(s.par_o, level)
    keys_o, keys = _gk(fg, ora, s, exps)
    ek = ora.EvaluationKey(s.sk, s.rng)
    ek.gk = dict(zip(exps, keys_o))
    w = s.rng.integers(0, s.t, n, dtype=np.uint64)
    ct = s.sk.encrypt(ora.Plaintext.encode(w, "poly", s.par_o), s.rng)
    got = fg.to_host(fg.expand(s.par, keys, fg.to_device(ct.to_array()), size))
    want = ek.expands(ct, size)
    for i in range(size):
        assert np.array_equal(got[i], want[i].to_array()), i
        m = s.sk.decrypt(ora.Ciphertext.from_array(s.par_o, got[i], 0)).decode("poly")
        assert int(m[0]) == int(w[i]) * (1 << level) % s.t


@pytest.mark.parametrize("n,L,count,groups", [(4096, 2, 5, 1), (16384, 6, 20, 3)])
def test_dot_product(fg, ora, cuda, n, L, count, groups):
    s = Setup(fg, ora, n, L, 65537, seed=count + groups)
    vals, cts = s.encrypt(count * groups)
    pv = s.rng.integers(0, 65537, (count, n), dtype=np.uint64)
    pts = fg.plaintext_encode(s.par, 0, fg.to_device(pv))
    arr = np.stack([c.to_array() for c in cts]).reshape(groups, count, 2, L, n)
    got = fg.to_host(fg.dot_product_scalar(s.par, 0, fg.to_device(arr), pts))
    ctx = s.par_o.context_at_level(0)
    pts_o = [ora.Poly.from_u64(ctx, ora.Plaintext.encode(pv[c], "simd", s.par_o).value).into_ntt() for c in range(count)]
    for g in range(groups):
        want = ora.dot_product_scalar(cts[g * count:(g + 1) * count], pts_o)
        assert np.array_equal(got[g], want.to_array())
        dec = [int(x) for x in s.decrypt(got[g], 0)]
        expect = [sum(int(vals[g * count + c][i]) * int(pv[c][i]) for c in range(count)) % 65537 for i in range(n)]
        assert dec == expect
