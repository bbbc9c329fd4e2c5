"""The allocation-free relinearization entry point.

Some callers of this library cannot let it allocate device memory (stream
capture, allocation-free serving loops, applications owning all device
memory). fheg_relinearize_noalloc serves them with a fixed scratch array
inside the library. This test calls it through the C ABI and checks that two
calls in a row give exactly what fheg_relinearize gives. It lives in its own
file, collected last, so a run that stops at the first failure has already run
every other test."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ct3_batch(ora, par, sk, rng, count, level=0):
    cts = []
    for _ in range(count):
        vals = rng.integers(0, par.plaintext, par.degree, dtype=np.uint64)
        a = sk.encrypt(ora.Plaintext.encode(vals, "simd", par, level), rng)
        b = sk.encrypt(ora.Plaintext.encode(vals, "simd", par, level), rng)
        cts.append((a * b).to_array())
    return np.stack(cts)


# (ciphertext level, key level): a key at the ciphertext's level, and a key one
# level below it, whose key switch also switches down.
@pytest.mark.parametrize("ct_level,key_level", [(0, 0), (1, 0)])
def test_relinearize_noalloc_matches_relinearize(fg, ora, cuda, ct_level, key_level):
    rng = np.random.default_rng(404 + ct_level)
    par_o = ora.BfvParameters(4096, 65537, moduli_sizes=[62, 62, 62])
    sk = ora.SecretKey.random(par_o, rng)
    rk_o = ora.RelinearizationKey(sk, rng, ct_level, key_level)
    par = fg.BfvParameters(4096, par_o.moduli, 65537)
    rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array(), ct_level, key_level)
    lib = fg.lib()
    stream = cuda.cuda.current_stream().cuda_stream
    for call in range(2):
        ct3 = fg.to_device(_ct3_batch(ora, par_o, sk, rng, 3, ct_level))
        expected = rk.relinearizes(ct3)
        out = fg.empty(expected.shape)
        fg.check(lib.fheg_relinearize_noalloc(rk._h, ct3.data_ptr(), out.data_ptr(), 3, stream))
        cuda.cuda.synchronize()
        assert np.array_equal(fg.to_host(out), fg.to_host(expected)), f"call {call}"


def test_relinearize_noalloc_rejects_oversized_batches(fg, ora, cuda):
    rng = np.random.default_rng(405)
    par_o = ora.BfvParameters(16384, 65537, moduli_sizes=[62] * 6)
    sk = ora.SecretKey.random(par_o, rng)
    rk_o = ora.RelinearizationKey(sk, rng)
    par = fg.BfvParameters(16384, par_o.moduli, 65537)
    rk = fg.RelinearizationKey(par, rk_o.ksk.c0_array(), rk_o.ksk.c1_array())
    # 8 * count * L * N * (1 + L) = 5.5 MB per ciphertext here: 4 exceed 16 MiB.
    ct3 = fg.empty((4, 3, 6, 16384))
    out = fg.empty((4, 2, 6, 16384))
    status = fg.lib().fheg_relinearize_noalloc(rk._h, ct3.data_ptr(), out.data_ptr(), 4, None)
    assert status == fg.ERR_INVALID_ARGUMENT
    assert b"scratch" in fg.lib().fheg_last_error()
