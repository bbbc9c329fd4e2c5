"""Generates the golden fixtures of this directory from the CPU oracle.

    python tests/golden/make_golden.py

Each fixture is a seeded case small enough to commit: inputs and the outputs
the oracle (the restatement of fhe.rs under oracle/) gives for them. The GPU
tests compare the CUDA path with these files without running the oracle, and
tests/test_golden.py regenerates every case and checks that the oracle still
produces the same bytes. The fhe.rs reference itself (Rust) cannot be run
here, so these are not outputs of fhe.rs; what pins the oracle to fhe.rs is
tests/test_oracle_pins.py.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _ntt_case(ora, n, sizes, seed):
    rng = np.random.default_rng(seed)
    moduli = []
    for bits in sizes:
        ub = 1 << bits
        while True:
            p = ora.generate_prime(bits, 2 * n, ub)
            ub = p
            if p not in moduli:
                moduli.append(p)
                break
    roots = [ora.ntt_operator(p, n).omega for p in moduli]
    x = np.stack([rng.integers(0, p, n, dtype=np.uint64) for p in moduli])
    fwd, lazy = x.copy(), x.copy()
    for j, p in enumerate(moduli):
        op = ora.ntt_operator(p, n)
        op.forward(fwd[j])
        op.forward_vt_lazy(lazy[j])
    back = fwd.copy()
    for j, p in enumerate(moduli):
        ora.ntt_operator(p, n).backward(back[j])
    return {"moduli": np.array(moduli, dtype=np.uint64), "roots": np.array(roots, dtype=np.uint64), "x": x,
            "forward": fwd, "forward_lazy": lazy, "backward": back}


def _scaler_case(ora, seed):
    """RnsScaler from 4 moduli to 3 (different contexts) by num/den, applied
    to every coefficient of a power-basis polynomial (n = 16)."""
    rng = np.random.default_rng(seed)
    n = 16
    frm = ora.BfvParameters.generate_moduli([62, 62, 62, 62], n)
    to = ora.BfvParameters.generate_moduli([50, 50, 50], n)
    num, den = 65537 * 1009, int(ora.RnsContext(frm).modulus() // 3)
    x = np.stack([rng.integers(0, p, n, dtype=np.uint64) for p in frm])
    s = ora.RnsScaler(ora.RnsContext(frm), ora.RnsContext(to), ora.ScalingFactor(num, den))
    y = s.scale_columns(x, 0, len(to))
    return {"from": np.array(frm, dtype=np.uint64), "to": np.array(to, dtype=np.uint64),
            "num": np.array([num & (2**64 - 1), num >> 64], dtype=np.uint64),
            "den": np.array([(den >> (64 * k)) & (2**64 - 1) for k in range(4)], dtype=np.uint64), "x": x, "y": y}


def _bfv_case(ora, n, L, t, seed):
    """Multiplicator::default with relinearization, a row rotation, a column
    rotation, a switch-down and an addition on seeded encryptions."""
    rng = np.random.default_rng(seed)
    par = ora.BfvParameters(n, t, moduli_sizes=[62] * L)
    sk = ora.SecretKey.random(par, rng)
    rk = ora.RelinearizationKey(sk, rng)
    vals = [rng.integers(0, t, n, dtype=np.uint64) for _ in range(2)]
    cts = [sk.encrypt(ora.Plaintext.encode(v, "simd", par), rng) for v in vals]
    prod = ora.Multiplicator.default(rk).multiply(cts[0], cts[1])
    g_row = ora.GaloisKey(sk, 2 * n - 1, 0, 0, rng)
    e_col = ora.rotation_exponent(par, 1)
    g_col = ora.GaloisKey(sk, e_col, 0, 0, rng)
    return {"moduli": np.array(par.moduli, dtype=np.uint64), "t": np.array([t], dtype=np.uint64),
            "sk": np.asarray(sk.coeffs, dtype=np.int64), "values": np.stack(vals),
            "ct0": cts[0].to_array(), "ct1": cts[1].to_array(),
            "rk_c0": rk.ksk.c0_array(), "rk_c1": rk.ksk.c1_array(), "product": prod.to_array(),
            "row_exponent": np.array([2 * n - 1], dtype=np.uint64),
            "row_c0": g_row.ksk.c0_array(), "row_c1": g_row.ksk.c1_array(),
            "row_rotated": g_row.relinearize(cts[0]).to_array(),
            "col_exponent": np.array([e_col], dtype=np.uint64),
            "col_c0": g_col.ksk.c0_array(), "col_c1": g_col.ksk.c1_array(),
            "col_rotated": g_col.relinearize(cts[1]).to_array(),
            "switched_down": cts[0].copy().switch_down().to_array(),
            "sum": (cts[0] + cts[1]).to_array()}


CASES = {
    "ntt_n16": lambda ora: _ntt_case(ora, 16, [62, 62, 50], 11),
    "ntt_n1024": lambda ora: _ntt_case(ora, 1024, [62, 40], 12),
    "ntt_n4096": lambda ora: _ntt_case(ora, 4096, [62], 13),
    "scaler_n16": lambda ora: _scaler_case(ora, 14),
    "bfv_n16_l3": lambda ora: _bfv_case(ora, 16, 3, 1153, 15),
    "bfv_n256_l2": lambda ora: _bfv_case(ora, 256, 2, 65537, 16),
}


def generate(name: str) -> dict:
    from oracle import build as oracle_build
    from oracle import ora

    oracle_build.build()
    return CASES[name](ora)


def path(name: str) -> str:
    return os.path.join(HERE, name + ".npz")


def load(name: str) -> dict:
    with np.load(path(name)) as f:
        return {k: f[k] for k in f.files}


def main():
    for name in CASES:
        np.savez_compressed(path(name), **generate(name))
        print(name, os.path.getsize(path(name)), "bytes")


if __name__ == "__main__":
    main()
