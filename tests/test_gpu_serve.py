"""Serving runtime: a mix of mul+relin, rotations, additions and
switch-downs at several levels, submitted together, gives each request the
result it gets alone and the oracle's result; HBM-budget admission and
bounded waits."""

import numpy as np
import pytest

from test_gpu_bfv import Setup

pytestmark = pytest.mark.gpu


def _pinned_like(fg, arr):
    """A numpy view of a pinned host buffer holding `arr`."""
    import torch

    t = torch.empty(arr.shape, dtype=torch.int64, pin_memory=True)
    v = t.numpy().view(np.uint64)
    v[...] = arr
    return t, v


def _mix(fg, ora, s, levels=(0, 1), per_kind=3):
    """Requests (kind, args, expected) with oracle results."""
    reqs = []
    rk_o, rk = s.rk(0)
    mult_o = ora.Multiplicator.default(rk_o)
    mult = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(2 * per_kind, level=0)
    for i in range(per_kind):
        a, b = cts[2 * i], cts[2 * i + 1]
        reqs.append(("mul", (mult, a.to_array(), b.to_array()), mult_o.multiply(a, b).to_array()))
    keys = {}
    for lvl in levels:
        for j, e in enumerate([2 * s.n - 1, ora.rotation_exponent(s.par_o, 1 + lvl)]):
            gk_o = ora.GaloisKey(s.sk, e, lvl, lvl, s.rng)
            keys[(lvl, j)] = (gk_o, fg.GaloisKey(s.par, e, gk_o.ksk.c0_array(), gk_o.ksk.c1_array(), lvl, lvl))
        _, cl = s.encrypt(3 * per_kind, level=lvl)
        for i in range(per_kind):
            gk_o, gk = keys[(lvl, i % 2)]
            reqs.append(("rot", (gk, cl[i].to_array()), gk_o.relinearize(cl[i]).to_array()))
            x, y = cl[per_kind + i], cl[2 * per_kind + i]
            reqs.append(("add", (s.par, lvl, x.to_array(), y.to_array()), (x + y).to_array()))
            reqs.append(("down", (s.par, lvl, y.to_array()), y.copy().switch_down().to_array()))
    return reqs, (mult, keys)


def _submit(srv, kind, args, out=None):
    if kind == "mul":
        return srv.submit_mul_relin(*args, out=out)
    if kind == "rot":
        return srv.submit_rotate(*args, out=out)
    if kind == "add":
        return srv.submit_add(*args, out=out)
    return srv.submit_switch_down(*args, out=out)


@pytest.mark.parametrize("n,L", [(4096, 3), (16384, 4)])
def test_mix_equals_alone_and_oracle(fg, ora, cuda, n, L):
    s = Setup(fg, ora, n, L, 65537, seed=500 + n)
    reqs, _keep = _mix(fg, ora, s)
    order = np.random.default_rng(3).permutation(len(reqs))
    with fg.Server(hbm_budget_bytes=1 << 30, streams=3, max_batch=8) as srv:
        # In the mix: everything submitted at once, in a shuffled order, half
        # of the outputs pinned (direct copies) and half pageable (staged).
        pinned, ids = {}, {}
        for k, idx in enumerate(order):
            kind, args, want = reqs[idx]
            out = None
            if k % 2:
                t, out = _pinned_like(fg, np.zeros_like(want))
                pinned[idx] = t
            ids[idx] = _submit(srv, kind, args, out)
        mixed = {idx: srv.wait(rid) for idx, rid in ids.items()}
        st = srv.stats()
        assert st["completed"] == len(reqs)
        assert st["batches"] < len(reqs)  # requests did share launches
        # Alone: one request at a time.
        for idx, (kind, args, want) in enumerate(reqs):
            alone = srv.wait(_submit(srv, kind, args))
            assert np.array_equal(mixed[idx], alone), f"request {idx} ({kind})"
            assert np.array_equal(alone, want), f"request {idx} ({kind}) vs oracle"


def test_budget_admission(fg, ora, cuda):
    """A budget that holds one mul+relin at a time still completes every
    request; a request larger than the whole budget fails with
    FHEG_ERR_BUDGET and does not block the others."""
    s = Setup(fg, ora, 16384, 4, 65537, seed=61)
    rk_o, rk = s.rk(0)
    mult, mult_o = fg.Multiplicator.default(rk), ora.Multiplicator.default(rk_o)
    _, cts = s.encrypt(8)
    one = 8 * 2 * 4 * 16384  # bytes of one ciphertext (1 MiB)
    # one pair needs 3 MiB of inputs and output plus ~13 MiB of scratch: 24 MiB
    # holds one pair but not two
    budget = 24 * one
    with fg.Server(hbm_budget_bytes=budget, streams=2, max_batch=8) as srv:
        ids = [srv.submit_mul_relin(mult, cts[2 * i].to_array(), cts[2 * i + 1].to_array()) for i in range(4)]
        outs = [srv.wait(r) for r in ids]
        st = srv.stats()
        assert st["batches"] == 4 and st["peak_bytes"] <= budget
        for i in range(4):
            assert np.array_equal(outs[i], mult_o.multiply(cts[2 * i], cts[2 * i + 1]).to_array())
    with fg.Server(hbm_budget_bytes=4 * one, streams=2, max_batch=8) as srv:  # an addition fits
        big = srv.submit_mul_relin(mult, cts[0].to_array(), cts[1].to_array())
        small = srv.submit_add(s.par, 0, cts[2].to_array(), cts[3].to_array())
        with pytest.raises(fg.FhegError) as e:
            srv.wait(big)
        assert e.value.code == fg.ERR_BUDGET
        assert np.array_equal(srv.wait(small), (cts[2] + cts[3]).to_array())


def test_bounded_wait_and_errors(fg, ora, cuda):
    s = Setup(fg, ora, 16384, 6, 65537, seed=62)
    rk_o, rk = s.rk(0)
    mult = fg.Multiplicator.default(rk)
    _, cts = s.encrypt(2)
    a, b = cts[0].to_array(), cts[1].to_array()
    with fg.Server(hbm_budget_bytes=1 << 30, streams=1, max_batch=64) as srv:
        ids = [srv.submit_mul_relin(mult, a, b) for _ in range(32)]
        with pytest.raises(fg.FhegError) as e:
            srv.wait(ids[-1], timeout_ms=0)
        assert e.value.code == fg.ERR_TIMEOUT
        outs = [srv.wait(r) for r in ids]
        assert all(np.array_equal(o, outs[0]) for o in outs)
        t0, t1, t2 = srv.times(ids[-1])
        assert t0 <= t1 <= t2
        srv.release(ids[-1])
        # invalid requests are rejected at submission
        with pytest.raises(fg.FhegError):
            srv.submit_switch_down(s.par, 5, a[:, :1])  # no level below the last
        with pytest.raises(fg.FhegError):
            srv.submit_mul_relin(mult, a[:1], b)  # one part only
