"""RGSW external product on the GPU (rgsw_ciphertext.rs:123-160): bit-exact
against the oracle's two key switches and their sum, and decrypting to the
slotwise product as the reference's own test checks (rgsw_ciphertext.rs:172-210)."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


def _rgsw(fg, ora, s, values, level):
    pt = ora.Plaintext.encode(values, "simd", s.par_o, level)
    r = ora.RGSWCiphertext(s.sk, pt, s.rng)
    dev = fg.RGSWCiphertext(s.par, r.ksk0.c0_array(), r.ksk0.c1_array(), r.ksk1.c0_array(), r.ksk1.c1_array(),
                            level)
    return r, dev


@pytest.mark.parametrize("n,L,t,level,B", [(16, 2, 1153, 0, 3), (16, 8, 1153, 0, 2), (4096, 3, 65537, 1, 2),
                                           (16384, 6, 65537, 0, 2), (32768, 4, 65537, 0, 1)])
def test_external_product_matches_oracle(fg, ora, cuda, n, L, t, level, B):
    s = Setup(fg, ora, n, L, t, seed=5 * n + L, level=level)
    v2 = s.rng.integers(0, t, n, dtype=np.uint64)
    r_o, r = _rgsw(fg, ora, s, v2, level)
    vals, cts = s.encrypt(B)
    arr = np.stack([c.to_array() for c in cts])
    got = fg.to_host(r.external_product(fg.to_device(arr)))
    assert got.shape == (B, 2, L - level, n)
    for b in range(B):
        want = r_o.external_product(cts[b]).to_array()
        assert np.array_equal(got[b], want), b
        assert list(s.decrypt(got[b], level)) == s.product(vals[b], v2)
    # Mul<&Ciphertext> for &RGSWCiphertext, and the output over the input.
    dev = fg.to_device(arr)
    assert np.array_equal(fg.to_host(r * dev), got)
    r.external_product(dev, out=dev)
    assert np.array_equal(fg.to_host(dev), got)


def test_external_product_errors(fg, ora, cuda):
    s = Setup(fg, ora, 16, 3, 1153, seed=9)
    v2 = s.rng.integers(0, 1153, 16, dtype=np.uint64)
    _, r = _rgsw(fg, ora, s, v2, 0)
    _, cts = s.encrypt(1)
    ct = cts[0].to_array()
    with pytest.raises(fg.FhegError) as e:
        r.external_product(fg.to_device(np.stack([ct, ct])[:, :1]))  # one part
    assert e.value.code == fg.ERR_WRONG_PARTS
    with pytest.raises(fg.FhegError) as e:
        r.external_product(fg.to_device(ct[None, :, :2]))  # another level
    assert e.value.code == fg.ERR_INVALID_LEVEL
    k = np.zeros((3, 3, 16), dtype=np.uint64)
    with pytest.raises(fg.FhegError) as e:
        fg.RGSWCiphertext(s.par, k, k, k, k, level=3)
    assert e.value.code == fg.ERR_INVALID_LEVEL
    one = Setup(fg, ora, 16, 1, 1153, seed=1)
    k1 = np.zeros((1, 1, 16), dtype=np.uint64)
    with pytest.raises(fg.FhegError) as e:
        fg.RGSWCiphertext(one.par, k1, k1, k1, k1)
    assert e.value.code == fg.ERR_UNSUPPORTED
