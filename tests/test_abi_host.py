"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, and its host-side precomputation (an independent C++ restatement)
equals the oracle's. No kernels are launched here."""

import ctypes
import re

import numpy as np
import pytest


def _declared_symbols(header_path):
    text = open(header_path).read()
    return sorted(set(re.findall(r"FHEG_API\s+[^;{(]*?\b(fheg_\w+)\s*\(", text)))


def test_library_exports_header_symbols(fg):
    names = _declared_symbols(fg.HEADER_PATH)
    assert len(names) >= 30
    lib = ctypes.CDLL(fg.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(fg):
    assert fg.lib().fheg_status_string(0) == b"ok"
    assert fg.lib().fheg_version().startswith(b"fheg")


def test_generate_prime_matches_oracle(fg, ora):
    ub = ((1 << 64) - 1) >> 2
    for _ in range(20):
        p = fg.generate_prime(62, 2 * 1048576, ub)
        assert p == ora.generate_prime(62, 2 * 1048576, ub)
        ub = p
    assert fg.generate_prime(10, 2048, 1 << 10) is None
    assert fg.generate_prime(11, 16, 1033) is None
    # the moduli the BFV configurations use (62-bit, 2N = 2^15)
    ub = 1 << 62
    for _ in range(13):
        p = fg.generate_prime(62, 2 * 16384, ub)
        assert p == ora.generate_prime(62, 2 * 16384, ub)
        ub = p


@pytest.mark.parametrize("p,n", [(1153, 32), (4611686018326724609, 1024), (4611686018427322369, 4096),
                                 (65537, 16384), (4611686018427322369, 16384)])
def test_default_root_and_tables_match_oracle(fg, ora, p, n):
    root = fg.ntt_default_root(p, n)
    op = ora.NttOperator(ora.Modulus(p), n)
    assert root == op.omega
    (w, ws, zi, zis), (ninv, ninvs) = fg.ntt_tables_host(p, n)
    assert np.array_equal(w, op.omegas) and np.array_equal(ws, op.omegas_shoup)
    assert np.array_equal(zi, op.zetas_inv) and np.array_equal(zis, op.zetas_inv_shoup)
    assert (ninv, ninvs) == (op.size_inv, op.size_inv_shoup)


def test_injected_root_is_validated(fg):
    p, n = 4611686018326724609, 1024
    root = fg.ntt_default_root(p, n)
    (w, _, _, _), _ = fg.ntt_tables_host(p, n, pow(root, 3, p))
    assert int(w[1]) == pow(pow(root, 3, p), n // 2, p)
    with pytest.raises(fg.FhegError):
        fg.ntt_tables_host(p, n, 2)  # not a primitive 2n-th root


@pytest.mark.parametrize("frm,to,n,d", [
    ([4, 4611686018326724609, 1153], [4, 4611686018326724609, 1153], 3, 1001),
    ([4, 4611686018326724609, 1153], [4611686018309947393, 4611686018282684417], 4611686018326724610, 4),
    ([4611686018282684417, 4611686018326724609, 4611686018309947393],
     [4611686018282684417, 4611686018309947393, 4611686018257518593], 1000, 101),
])
def test_rns_scaler_constants_match_oracle(fg, ora, frm, to, n, d):
    got = fg.rns_scaler_constants_host(frm, to, n, d)
    s = ora.RnsScaler(ora.RnsContext(frm), ora.RnsContext(to), ora.ScalingFactor(n, d))
    assert got["theta_garner_shift"] == s.theta_garner_shift
    assert got["theta_gamma"] == (s.theta_gamma[0], s.theta_gamma[1], bool(s.theta_gamma[2]))
    for k in ("gamma", "gamma_shoup", "omega", "omega_shoup", "theta_omega_lo", "theta_omega_hi",
              "theta_omega_sign", "theta_garner_lo", "theta_garner_hi"):
        assert np.array_equal(got[k], getattr(s, k)), k


def test_mul_scaler_constants_match_oracle(fg, ora):
    """The t/Q scale-down of the N=2^14, L=6 multiplication (13 -> 6 moduli)."""
    par = ora.BfvParameters(16384, 65537, moduli_sizes=[62] * 6)
    ext = ora.Multiplicator.default_extended_basis(par, 0)
    q = par.context_at_level(0).modulus()
    got = fg.rns_scaler_constants_host(ext, par.moduli, 65537, q)
    s = ora.RnsScaler(ora.RnsContext(ext), ora.RnsContext(par.moduli), ora.ScalingFactor(65537, q))
    assert got["theta_garner_shift"] == s.theta_garner_shift
    for k in ("gamma", "omega", "omega_shoup", "theta_omega_lo", "theta_omega_hi", "theta_garner_lo",
              "theta_garner_hi"):
        assert np.array_equal(got[k], getattr(s, k)), k


def test_ntt_plan_validation(fg):
    """Plan entries are checked on the host: defaults single pass up to 2^12
    and 2^12 blocks above, in clusters at 2^13 and 2^14; blocks of 2^12..2^14
    with at most four strided stages."""
    for logn in range(3, 17):
        assert fg.ntt_plan_get(logn) == (logn if logn <= 12 else 12)
        assert fg.ntt_cluster_get(logn) == (logn in (13, 14))
    for logn, bl in [(12, 11), (14, 15), (15, 15), (16, 11), (17, 14), (11, 12)]:
        with pytest.raises(fg.FhegError):
            fg.ntt_plan_set(logn, bl)
    fg.ntt_plan_set(14, 14)
    assert fg.ntt_plan_get(14) == 14
    fg.ntt_plan_set(14, 12)
    assert fg.ntt_plan_get(14) == 12


def test_no_device_fails_loudly(fg):
    """Without a CUDA device every entry point that needs one returns a CUDA
    error status (no silent host fallback)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(fg.FhegError) as e:
        fg.Context([4611686018427322369], 4096)
    assert e.value.code == fg.ERR_CUDA
    ptr = ctypes.c_void_p()
    assert fg.lib().fheg_device_alloc(1 << 20, ctypes.byref(ptr)) == fg.ERR_CUDA
    fg.ntt_prefetch_set(False)  # host-only settings still work


def test_c_client_compiles_and_links(fg, tmp_path):
    """include/fheg.h is valid C99 (what a cgo / bindgen / ctypes binding
    parses) and a C program links against libfheg.so and calls it."""
    import os
    import shutil
    import subprocess

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib_dir = os.path.dirname(fg.build())
    exe = str(tmp_path / "abi_client")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(root, "include"),
           os.path.join(root, "tests", "c", "abi_client.c"), "-L", lib_dir, "-lfheg", "-Wl,-rpath," + lib_dir,
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("ok 4611686018427322369")
