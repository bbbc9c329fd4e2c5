"""The committed golden fixtures (tests/golden/*.npz): the oracle still
produces them byte for byte (CPU), the fixtures decrypt to what they should
(CPU), and the CUDA path reproduces them from the files alone (GPU)."""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402

NAMES = sorted(make_golden.CASES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_fixture(ora, name):
    want = make_golden.load(name)
    got = make_golden.generate(name)
    assert sorted(got) == sorted(want)
    for k in want:
        assert got[k].dtype == want[k].dtype and np.array_equal(got[k], want[k]), f"{name}:{k}"


@pytest.mark.parametrize("name", ["bfv_n16_l3", "bfv_n256_l2"])
def test_fixture_decrypts(ora, name):
    g = make_golden.load(name)
    n, t = g["ct0"].shape[-1], int(g["t"][0])
    par = ora.BfvParameters(n, t, moduli=[int(q) for q in g["moduli"]])
    sk = ora.SecretKey(par, g["sk"])

    def dec(arr, level=0):
        return [int(x) for x in sk.decrypt(ora.Ciphertext.from_array(par, arr, level)).decode("simd")]

    a, b = [int(x) for x in g["values"][0]], [int(x) for x in g["values"][1]]
    assert dec(g["ct0"]) == a and dec(g["ct1"]) == b
    assert dec(g["product"]) == [x * y % t for x, y in zip(a, b)]
    assert dec(g["sum"]) == [(x + y) % t for x, y in zip(a, b)]
    assert dec(g["switched_down"], 1) == a
    # row rotation swaps the two rows of the SIMD matrix (evaluation_key.rs:572-610)
    h = n // 2
    assert dec(g["row_rotated"]) == a[h:] + a[:h]
    # column rotation by one step rotates each row left by one (evaluation_key.rs:612-675)
    assert dec(g["col_rotated"]) == b[1:h] + b[:1] + b[h + 1:] + b[h:h + 1]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ntt_n16", "ntt_n1024", "ntt_n4096"])
def test_gpu_ntt_matches_fixture(fg, cuda, name):
    g = make_golden.load(name)
    n = g["x"].shape[-1]
    ctx = fg.Context([int(p) for p in g["moduli"]], n, roots=[int(r) for r in g["roots"]])
    x = fg.to_device(g["x"][None])
    fg.ntt_forward(ctx, x)
    assert np.array_equal(fg.to_host(x)[0], g["forward"])
    y = fg.to_device(g["x"][None])
    fg.ntt_forward(ctx, y, lazy=True)
    assert np.array_equal(fg.to_host(y)[0], g["forward_lazy"])
    z = fg.to_device(g["forward"][None])
    fg.ntt_backward(ctx, z)
    assert np.array_equal(fg.to_host(z)[0], g["backward"])


@pytest.mark.gpu
def test_gpu_scaler_matches_fixture(fg, cuda):
    g = make_golden.load("scaler_n16")
    n = g["x"].shape[-1]
    frm = fg.Context([int(p) for p in g["from"]], n)
    to = fg.Context([int(p) for p in g["to"]], n)
    num = sum(int(w) << (64 * k) for k, w in enumerate(g["num"]))
    den = sum(int(w) << (64 * k) for k, w in enumerate(g["den"]))
    s = fg.Scaler(frm, to, fg.ScalingFactor(num, den))
    out = fg.to_host(s.scale(fg.to_device(g["x"][None]), 0))[0]
    assert np.array_equal(out, g["y"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bfv_n16_l3", "bfv_n256_l2"])
def test_gpu_bfv_matches_fixture(fg, cuda, name):
    g = make_golden.load(name)
    n, t = g["ct0"].shape[-1], int(g["t"][0])
    par = fg.BfvParameters(n, [int(q) for q in g["moduli"]], t)
    rk = fg.RelinearizationKey(par, g["rk_c0"], g["rk_c1"])
    ct0, ct1 = fg.to_device(g["ct0"][None]), fg.to_device(g["ct1"][None])
    prod = fg.Multiplicator.default(rk).multiply(ct0, ct1)
    assert np.array_equal(fg.to_host(prod)[0], g["product"])
    row = fg.GaloisKey(par, int(g["row_exponent"][0]), g["row_c0"], g["row_c1"])
    assert np.array_equal(fg.to_host(row.relinearize(ct0))[0], g["row_rotated"])
    col = fg.GaloisKey(par, int(g["col_exponent"][0]), g["col_c0"], g["col_c1"])
    assert np.array_equal(fg.to_host(col.relinearize(ct1))[0], g["col_rotated"])
    assert np.array_equal(fg.to_host(fg.ciphertext_add(par, 0, ct0, ct1))[0], g["sum"])
    assert np.array_equal(fg.to_host(fg.ciphertext_switch_down(par, 0, ct0.clone()))[0], g["switched_down"])
