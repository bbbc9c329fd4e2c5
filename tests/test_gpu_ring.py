"""GPU ring operations (fhe-math rq) bit-exact against the oracle: element-wise
ops, substitution, switch-down and the RNS scaler (rq::Scaler)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q = [4611686018282684417, 4611686018326724609, 4611686018309947393]
P = [4611686018282684417, 4611686018309947393, 4611686018257518593]
MODULI = [1153, 4611686018326724609, 4611686018309947393, 4611686018232352769, 4611686018171535361]


def _rand(rng, moduli, n, B):
    return np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli]) for _ in range(B)])


def test_poly_ops(fg, ora, cuda):
    rng = np.random.default_rng(1)
    n, B = 1 << 12, 3
    ctx_o = ora.Context(Q, n)
    ctx = fg.Context(Q, n)
    a, b = _rand(rng, Q, n, B), _rand(rng, Q, n, B)
    ta, tb = fg.to_device(a), fg.to_device(b)
    for op in ("add", "sub", "mul", "neg"):
        got = fg.to_host(fg.poly_op(ctx, op, ta, tb))
        for k in range(B):
            pa = ora.Poly(ctx_o, a[k], ora.NTT)
            pb = ora.Poly(ctx_o, b[k], ora.NTT)
            want = {"add": lambda: pa + pb, "sub": lambda: pa - pb, "mul": lambda: pa * pb, "neg": lambda: -pa}[op]()
            assert np.array_equal(got[k], want.coefficients), op


@pytest.mark.parametrize("n", [16, 1 << 13, 1 << 15])
def test_substitute(fg, ora, cuda, n):
    rng = np.random.default_rng(2)
    moduli = [m for m in MODULI if ora.supports_ntt(m, n)] or [ora.generate_prime(62, 2 * n, 1 << 62)]
    ctx_o = ora.Context(moduli, n)
    ctx = fg.Context(moduli, n)
    a = _rand(rng, moduli, n, 2)
    for e in (3, 11, 2 * n - 1, pow(3, 7, 2 * n)):
        ex = ora.SubstitutionExponent(ctx_o, e)
        for rep in (ora.POWER_BASIS, ora.NTT):
            got = fg.to_host(fg.substitute(ctx, fg.to_device(a), e, 0 if rep == ora.POWER_BASIS else 1))
            for k in range(2):
                want = ora.Poly(ctx_o, a[k], rep).substitute(ex)
                assert np.array_equal(got[k], want.coefficients), (e, rep)


@pytest.mark.parametrize("n", [16, 1 << 14])
def test_switch_down(fg, ora, cuda, n):
    """rq/mod.rs:390-448 in power basis, and in Ntt through the power basis."""
    rng = np.random.default_rng(3)
    moduli = [m for m in MODULI if ora.supports_ntt(m, n)]
    if len(moduli) < 3:
        moduli, ub = [], 1 << 62
        while len(moduli) < 4:
            ub = ora.generate_prime(62, 2 * n, ub)
            moduli.append(ub)
    ctx_o = ora.Context(moduli, n)
    ctx = fg.Context(moduli, n)
    a = _rand(rng, moduli, n, 3)
    got = fg.to_host(fg.switch_down(ctx, fg.to_device(a), 0))
    for k in range(3):
        want = ora.Poly(ctx_o, a[k], ora.POWER_BASIS).switch_down()
        assert np.array_equal(got[k], want.coefficients)
    got = fg.to_host(fg.switch_down(ctx, fg.to_device(a), 1))
    for k in range(3):
        want = ora.Poly(ctx_o, a[k], ora.NTT).into_power_basis().switch_down().into_ntt()
        assert np.array_equal(got[k], want.coefficients)


@pytest.mark.parametrize("num,den", [(1, 1), (3, 1001), (4611686018326724610, 4), (1000, 101), (100, 2)])
def test_scaler(fg, ora, cuda, num, den):
    """rq/scaler.rs:52-126 in both representations, different contexts."""
    rng = np.random.default_rng(4)
    n = 1 << 12
    frm_o, to_o = ora.Context(Q, n), ora.Context(P, n)
    sc_o = ora.Scaler(frm_o, to_o, ora.ScalingFactor(num, den))
    sc = fg.Scaler(fg.Context(Q, n), fg.Context(P, n), fg.ScalingFactor(num, den))
    a = _rand(rng, Q, n, 2)
    for rep in (ora.POWER_BASIS, ora.NTT):
        got = fg.to_host(sc.scale(fg.to_device(a), 0 if rep == ora.POWER_BASIS else 1))
        for k in range(2):
            want = sc_o.scale(ora.Poly(frm_o, a[k], rep))
            assert np.array_equal(got[k], want.coefficients), rep


def _boundary_values(q_from, num, den, n, rng):
    """n coefficients in [0, Q) at the scaler's rounding boundaries
    (rns/scaler.rs:249-352): near 0, Q/2 and Q, where the CRT overflow
    estimate v rounds, and, for a factor num/den other than one, values
    where x * num / den is within a few units of a half-integer, where w
    rounds. Both sums then sit next to a rounding boundary, which is where a
    kernel that keeps only their high words must fall back to the exact sums."""
    vals = [0, 1, 2, 3, q_from - 1, q_from - 2, q_from - 3] + [q_from // 2 + d for d in range(-4, 5)]
    if num != den:
        top = num * q_from // den
        for u in rng.integers(0, 1 << 62, 64, dtype=np.uint64):
            m = (int(u) * top) >> 62  # spread over [0, top)
            x = ((2 * m + 1) * den) // (2 * num)
            vals += [x + d for d in range(-2, 3) if 0 <= x + d < q_from]
    vals = [v % q_from for v in vals]
    rng.shuffle(vals)
    return (vals * (n // len(vals) + 1))[:n]


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("setup", ["ring_3001", "ring_t_over_q", "mul_up_6", "mul_up_12", "mul_down_13", "mul_down_25"])
def test_scaler_rounding_boundaries(fg, ora, cuda, setup, tc):
    """Coefficients chosen at the rounding boundaries of RnsScaler::scale, in
    both representations, for generic and exact-count scaler kernels, with the
    exact counts' products on the tensor cores (tc) and on the CUDA cores: the
    results equal the oracle's exact big-integer computation."""
    default = fg.rns_tensor_get()
    fg.rns_tensor_set(tc)
    try:
        _scaler_boundaries(fg, ora, setup)
    finally:
        fg.rns_tensor_set(default)
    assert fg.rns_tensor_wait_failures() == 0


def _scaler_boundaries(fg, ora, setup):
    rng = np.random.default_rng(["ring_3001", "ring_t_over_q", "mul_up_6", "mul_up_12", "mul_down_13", "mul_down_25"].index(setup))
    n = 4096
    if setup.startswith("ring"):
        frm, to = Q, P
        num, den = (3, 1001) if setup == "ring_3001" else (65537, ora.RnsContext(Q).modulus())
    else:
        L = {"mul_up_6": 6, "mul_up_12": 12, "mul_down_13": 6, "mul_down_25": 12}[setup]
        n = 16384 if L == 6 else 32768
        par = ora.BfvParameters(n, 65537, moduli_sizes=[62] * L)
        ext = ora.Multiplicator.default_extended_basis(par, 0)
        if setup.startswith("mul_up"):
            frm, to, num, den = list(par.moduli), ext, 1, 1
        else:
            frm, to, num, den = ext, list(par.moduli), 65537, par.context_at_level(0).modulus()
    frm_o, to_o = ora.Context(frm, n), ora.Context(to, n)
    sc_o = ora.Scaler(frm_o, to_o, ora.ScalingFactor(num, den) if num != den else ora.ScalingFactor.one())
    sc = fg.Scaler(fg.Context(frm, n), fg.Context(to, n),
                   fg.ScalingFactor(num, den) if num != den else fg.ScalingFactor.one())
    pb = ora.Poly.from_biguints(frm_o, _boundary_values(frm_o.modulus(), num, den, n, rng))
    got = fg.to_host(sc.scale(fg.to_device(pb.coefficients[None]), 0))[0]
    assert np.array_equal(got, sc_o.scale(pb).coefficients)
    nt = pb.copy().into_ntt()
    got = fg.to_host(sc.scale(fg.to_device(nt.coefficients[None]), 1))[0]
    assert np.array_equal(got, sc_o.scale(nt).coefficients)


def _primes(ora, n, count, bits=62):
    out, ub = [], 1 << bits
    while len(out) < count:
        ub = ora.generate_prime(bits, 2 * n, ub)
        out.append(ub)
    return out


@pytest.mark.parametrize("F,T", [(12, 1), (12, 7), (12, 10), (12, 13), (13, 3), (13, 8), (13, 10), (25, 5), (25, 12),
                                 (25, 16)])
@pytest.mark.parametrize("factor", ["one", "t_over_q", "3_1001"])
def test_scaler_tensor_core_shapes(fg, ora, cuda, F, T, factor):
    """Scalers from 12, 13 and 25 source moduli (the tensor-core form; 13 into
    more than 8 targets takes the generic kernel; 25 has column sums above
    2^23) into 1 to 16 target moduli of mixed sizes, with and without the
    signed theta sum (factor one or not), over 64 or 128 tensor-memory
    columns: equal to the oracle in both representations and to the CUDA-core
    form."""
    n = 4096
    rng = np.random.default_rng(F * 100 + T)
    pool = _primes(ora, n, F + T, 62)
    frm = pool[:F]
    to = pool[F:F + T - T // 2] + _primes(ora, n, T // 2, 40)  # some targets near 2^40
    num, den = {"one": (1, 1), "t_over_q": (65537, ora.RnsContext(frm).modulus()), "3_1001": (3, 1001)}[factor]
    frm_o, to_o = ora.Context(frm, n), ora.Context(to, n)
    sc_o = ora.Scaler(frm_o, to_o, ora.ScalingFactor(num, den) if num != den else ora.ScalingFactor.one())
    sc = fg.Scaler(fg.Context(frm, n), fg.Context(to, n),
                   fg.ScalingFactor(num, den) if num != den else fg.ScalingFactor.one())
    a = _rand(rng, frm, n, 2)
    default = fg.rns_tensor_get()
    try:
        for rep in (ora.POWER_BASIS, ora.NTT):
            r = 0 if rep == ora.POWER_BASIS else 1
            fg.rns_tensor_set(True)
            got = fg.to_host(sc.scale(fg.to_device(a), r))
            fg.rns_tensor_set(False)
            assert np.array_equal(got, fg.to_host(sc.scale(fg.to_device(a), r)))
            for k in range(2):
                assert np.array_equal(got[k], sc_o.scale(ora.Poly(frm_o, a[k], rep)).coefficients), (rep, k)
    finally:
        fg.rns_tensor_set(default)
    assert fg.rns_tensor_wait_failures() == 0


@pytest.mark.parametrize("tc", [True, False])
@pytest.mark.parametrize("n,L", [(4096, 2), (8192, 3), (16384, 6)])
def test_mul_scalers(fg, ora, cuda, n, L, tc):
    """The Multiplicator's scalers: extension Q -> Q u P (factor one, common
    prefix) and t/Q scale-down Q u P -> Q, in Ntt representation, with the
    products on the tensor cores (tc) and on the CUDA cores."""
    default = fg.rns_tensor_get()
    fg.rns_tensor_set(tc)
    try:
        _mul_scalers(fg, ora, n, L)
    finally:
        fg.rns_tensor_set(default)
    assert fg.rns_tensor_wait_failures() == 0


def _mul_scalers(fg, ora, n, L):
    rng = np.random.default_rng(5)
    par = ora.BfvParameters(n, 65537, moduli_sizes=[62] * L)
    ext = ora.Multiplicator.default_extended_basis(par, 0)
    base_o, mul_o = par.context_at_level(0), ora.Context(ext, n)
    base, mul = fg.Context(par.moduli, n), fg.Context(ext, n)
    up_o = ora.Scaler(base_o, mul_o, ora.ScalingFactor.one())
    down_o = ora.Scaler(mul_o, base_o, ora.ScalingFactor(65537, base_o.modulus()))
    up = fg.Scaler(base, mul, fg.ScalingFactor.one())
    down = fg.Scaler(mul, base, fg.ScalingFactor(65537, base_o.modulus()))
    a = _rand(rng, par.moduli, n, 2)
    got = fg.to_host(up.scale(fg.to_device(a), 1))
    for k in range(2):
        assert np.array_equal(got[k], up_o.scale(ora.Poly(base_o, a[k], ora.NTT)).coefficients)
    b = _rand(rng, ext, n, 2)
    got = fg.to_host(down.scale(fg.to_device(b), 1))
    for k in range(2):
        assert np.array_equal(got[k], down_o.scale(ora.Poly(mul_o, b[k], ora.NTT)).coefficients)


@pytest.mark.parametrize("n", [16, 1 << 14])
def test_ntt_shoup_representation(fg, ora, cuda, n):
    """Representation::NttShoup (rq/mod.rs:37-47, 209-223): the Shoup plane
    equals the oracle's, the NttShoup product (rq/ops.rs:208-245) equals the
    oracle's, and representation 2 serializes through the power basis and
    substitutes like Ntt (rq/mod.rs:319-369)."""
    rng = np.random.default_rng(12)
    moduli = [m for m in MODULI if ora.supports_ntt(m, n)] or [ora.generate_prime(62, 2 * n, 1 << 62)]
    moduli = moduli + [ora.generate_prime(40, 2 * n, 1 << 40)]
    ctx_o, ctx = ora.Context(moduli, n), fg.Context(moduli, n)
    a, b = _rand(rng, moduli, n, 3), _rand(rng, moduli, n, 3)
    for k in range(3):  # extreme residues
        b[k, :, 0] = 0
        for i, m in enumerate(moduli):
            b[k, i, 1] = m - 1
    db = fg.to_device(b)
    bs = fg.compute_shoup(ctx, db)
    got_s = fg.to_host(bs)
    prod = fg.to_host(fg.mul_shoup(ctx, fg.to_device(a), db, bs))
    for k in range(3):
        po = ora.Poly(ctx_o, b[k].copy(), ora.NTT_SHOUP)
        po.compute_coefficients_shoup()
        assert np.array_equal(got_s[k], po.coefficients_shoup)
        want = ora.Poly(ctx_o, a[k].copy(), ora.NTT)
        want.mul_assign(po)
        assert np.array_equal(prod[k], want.coefficients)
    payload = fg.serialize(ctx, db, 2)
    host = payload.cpu().numpy()
    for k in range(3):
        pb = ora.Poly(ctx_o, b[k].copy(), ora.NTT).into_power_basis()
        assert bytes(host[k]) == ora.rq_payload(pb)
    assert np.array_equal(fg.to_host(fg.deserialize(ctx, payload, 2)), b)
    ex = ora.SubstitutionExponent(ctx_o, 3)
    sub = fg.to_host(fg.substitute(ctx, db, 3, 2))
    for k in range(3):
        assert np.array_equal(sub[k], ora.Poly(ctx_o, b[k], ora.NTT_SHOUP).substitute(ex).coefficients)


def test_scalar_mul(fg, ora, cuda):
    """MulAssign<&BigUint> (rq/ops.rs:297-352): limb j times scalar mod q_j."""
    n = 4096
    moduli = [ora.generate_prime(62, 2 * n, 1 << 62)]
    moduli.append(ora.generate_prime(62, 2 * n, moduli[-1]))
    moduli.append(ora.generate_prime(40, 2 * n, 1 << 40))
    ctx = fg.Context(moduli, n)
    rng = np.random.default_rng(8)
    x = np.stack([np.stack([rng.integers(0, q, n, dtype=np.uint64) for q in moduli]) for _ in range(3)])
    for scalar in (0, 1, 65537, (1 << 200) + 12345, int(np.prod([float(q) for q in moduli[:1]]))):
        got = fg.to_host(fg.scalar_mul(ctx, fg.to_device(x), scalar))
        for j, q in enumerate(moduli):
            s = scalar % q
            want = np.array([int(v) * s % q for v in x[:, j].ravel()], dtype=np.uint64).reshape(x[:, j].shape)
            assert np.array_equal(got[:, j], want), (scalar, j)


@pytest.mark.parametrize("n,bits", [(16, [62, 62, 40]), (4096, [62, 50]), (16384, [62] * 6)])
def test_serialize_matches_oracle(fg, ora, cuda, n, bits):
    """The Rq coefficient payload (rq/convert.rs:17-93) byte for byte, both
    representations, and back."""
    moduli = []
    for b in bits:
        ub = 1 << b
        while True:
            ub = ora.generate_prime(b, 2 * n, ub)
            if ub not in moduli:
                moduli.append(ub)
                break
    ctx = fg.Context(moduli, n)
    octx = ora.Context(moduli, n)
    rng = np.random.default_rng(n)
    x = np.stack([np.stack([rng.integers(0, m, n, dtype=np.uint64) for m in moduli]) for _ in range(3)])
    for rep, orep in ((0, ora.POWER_BASIS), (1, ora.NTT)):
        got = fg.serialize(ctx, fg.to_device(x), rep).cpu().numpy()
        assert got.shape == (3, fg.serialized_size(ctx))
        for b in range(3):
            want = ora.rq_payload(ora.Poly(octx, x[b].copy(), orep))
            assert bytes(got[b].tobytes()) == want, (rep, b)
        back = fg.to_host(fg.deserialize(ctx, fg.serialize(ctx, fg.to_device(x), rep), rep))
        assert np.array_equal(back, x), rep
