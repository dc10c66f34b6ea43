"""The 64-bit path (N=2048, Q=18014398509404161 < 2^54, BG=2^9 x 6, n=630)
against the oracle, bit-exact."""
import os
import sys

import numpy as np
import pytest

from conftest import random_gate_batch, x1_gate_batch

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


def test_wide_ntt(F, ctx1, keys1, cuda_ok):
    torch = cuda_ok
    o = keys1.oracle
    Q = keys1.P.Q
    a = np.random.default_rng(1).integers(0, Q, (5, 2048), dtype=np.uint64)
    a[0, :4] = [0, 1, Q - 1, Q // 2]
    d = dev(torch, a)
    ctx1.ntt_forward(d.data_ptr(), 5)
    torch.cuda.synchronize()
    assert np.array_equal(host(d), np.stack([o.ntt(x) for x in a]))
    ctx1.ntt_inverse(d.data_ptr(), 5)
    torch.cuda.synchronize()
    assert np.array_equal(host(d), a)


def test_wide_rlwe_mult_rgsw(F, ctx1, keys1, cuda_ok):
    torch = cuda_ok
    o = keys1.oracle
    Q = keys1.P.Q
    rng = np.random.default_rng(2)
    acc = rng.integers(0, Q, (3, 4096), dtype=np.uint64)
    acc[0] = Q - 1
    rgsw = rng.integers(0, Q, (3, 6 * 4 * 2048), dtype=np.uint64)
    out = torch.zeros((3, 4096), dtype=torch.int64, device="cuda")
    da, dr = dev(torch, acc), dev(torch, rgsw)
    ctx1.rlwe_mult_rgsw(da.data_ptr(), dr.data_ptr(), out.data_ptr(), 3)
    torch.cuda.synchronize()
    assert np.array_equal(host(out), np.stack([o.rlwe_mult_rgsw(acc[i], rgsw[i]) for i in range(3)]))


def test_wide_keyswitch(F, ctx1, keys1, cuda_ok):
    torch = cuda_ok
    o = keys1.oracle
    rl = np.random.default_rng(3).integers(0, keys1.P.Q, (2, 4096), dtype=np.uint64)
    dr = dev(torch, rl)
    out = torch.zeros((2, keys1.P.n + 1), dtype=torch.int64, device="cuda")
    ctx1.lwe_keyswitch_async(dr.data_ptr(), 2, out.data_ptr())
    ctx1.sync()
    assert np.array_equal(host(out), np.stack([o.lwe_keyswitch(r, keys1.kskey) for r in rl]))


def test_wide_bootstrap_all_gates(F, ctx1, keys1):
    x, y, g, c1, c2 = random_gate_batch(keys1, 12, seed=5, gates=[0, 1, 2, 3, 4, 5] * 2)
    out = ctx1.eval_bootstrap_batch(c1, c2, g)
    want, failed = keys1.oracle.eval_bootstrap_batch(c1, c2, g, keys1.btkey, keys1.kskey)
    assert failed == 0
    assert np.array_equal(out, want)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys1.decrypt(out), truth)


def test_wide_blind_rotate(F, ctx1, keys1, cuda_ok):
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys1, 2, seed=6)
    d1, d2, dg = dev(torch, c1), dev(torch, c2), torch.from_numpy(g).cuda()
    acc = torch.zeros((2, 4096), dtype=torch.int64, device="cuda")
    ctx1.blind_rotate_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 2, acc.data_ptr())
    ctx1.sync()
    got = host(acc)
    for i in range(2):
        want, steps = keys1.oracle.blind_rotate(c1[i], c2[i], int(g[i]), keys1.btkey)
        assert steps > 1150
        assert np.array_equal(got[i], want)


_want12 = {}


@pytest.mark.parametrize("pipes,window", [(1, -1), (1, 0), (2, -1), (3, -1), (3, 0), (3, 4)])
def test_wide_worker_shapes(F, ctx1, keys1, pipes, window):
    """Every launch shape of the 64-bit blind rotation (1, 2 or 3 workers per
    CTA sharing a group item by item; step window on and off) gives the
    oracle's words."""
    x, y, g, c1, c2 = random_gate_batch(keys1, 12, seed=9)
    if "w" not in _want12:
        want, failed = keys1.oracle.eval_bootstrap_batch(c1, c2, g, keys1.btkey, keys1.kskey)
        assert failed == 0
        _want12["w"] = want
    ctx1.set_option(F.OPT_BR_PIPES, pipes)
    ctx1.set_option(F.OPT_BR_WINDOW, window)
    try:
        out = ctx1.eval_bootstrap_batch(c1, c2, g)
        assert ctx1.device_status() == 0
    finally:
        ctx1.set_option(F.OPT_BR_PIPES, 0)
        ctx1.set_option(F.OPT_BR_WINDOW, -1)
    assert np.array_equal(out, _want12["w"])


def test_wide_several_rounds(F, ctx1, keys1):
    """A group cap of one gate per worker makes the 3-worker CTAs claim three
    rounds of groups (1000 gates, 152 CTAs of at most 3); every gate decrypts
    and a spread sample equals the oracle."""
    count = 1000
    x, y, g, c1, c2 = random_gate_batch(keys1, count, seed=31)
    ctx1.set_option(F.OPT_BR_GROUP, 1)
    ctx1.set_option(F.OPT_BR_PIPES, 3)
    try:
        out = ctx1.eval_bootstrap_batch(c1, c2, g)
        assert ctx1.device_status() == 0
    finally:
        ctx1.set_option(F.OPT_BR_GROUP, 0)
        ctx1.set_option(F.OPT_BR_PIPES, 0)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys1.decrypt(out), truth)
    idx = np.array([0, 1, 455, 456, 500, 912, 999])
    want, failed = keys1.oracle.eval_bootstrap_batch(c1[idx], c2[idx], g[idx], keys1.btkey, keys1.kskey)
    assert failed == 0
    assert np.array_equal(out[idx], want)


@pytest.mark.parametrize("pipes", [1, 2])
def test_wide_fpga_compat_mode(F, ctx1, keys1, pipes):
    """The no-skip issue order (myfpga.cpp:1200-1210) on the 64-bit path with
    one and two workers per CTA, against the oracle run the same way."""
    x, y, g, c1, c2 = random_gate_batch(keys1, 4, seed=41)
    ctx1.set_option(F.OPT_BR_PIPES, pipes)
    try:
        out = ctx1.eval_bootstrap_batch(c1, c2, g, flags=F.FLAG_FPGA_COMPAT)
    finally:
        ctx1.set_option(F.OPT_BR_PIPES, 0)
    want, failed = keys1.oracle.eval_bootstrap_batch(c1, c2, g, keys1.btkey, keys1.kskey, fpga_compat=True)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("pipes", [1, 2])
def test_wide_fpga_x1_mode(F, ctx1, keys1, pipes):
    """The issue order of fpga_eval_bootstrap_x1 (myfpga.cpp:1037-1046) on the
    64-bit path with one and two workers per CTA, against the oracle."""
    x, y, g, c1, c2, zero = x1_gate_batch(keys1, 4, seed=43)
    ctx1.set_option(F.OPT_BR_PIPES, pipes)
    try:
        out = ctx1.eval_bootstrap_batch(c1, c2, g, flags=F.FLAG_FPGA_X1)
    finally:
        ctx1.set_option(F.OPT_BR_PIPES, 0)
    want, failed = keys1.oracle.eval_bootstrap_batch(c1, c2, g, keys1.btkey, keys1.kskey, fpga_compat=2)
    assert failed == 0
    assert np.array_equal(out, want)


@pytest.mark.parametrize("count", [40, 341, 2048, 4000])
def test_wide_tiled_keyswitch_equals_per_gate(F, ctx1, keys1, cuda_ok, count):
    """The tiled 64-bit LWE key switch (gate blocks sharing each key row group
    through shared memory; from two gates per SM by default) against the
    one-CTA-per-gate kernel on the same blind-rotation outputs: forced on 40
    gates (one gate per warp, a partial last block), then 341 (two per warp),
    2048 (nine per warp, the 2048-gate configuration's shape) and 4000 (16 per
    warp, more CTAs than SMs); a few gates also against the oracle. Integer
    words: bit-exact."""
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys1, count, seed=181 + count)
    d1, d2, dg = dev(torch, c1), dev(torch, c2), torch.from_numpy(g).cuda()
    tiled, per_gate = torch.zeros_like(d1), torch.zeros_like(d1)
    try:
        ctx1.set_option(F.OPT_KS_TILED, 1)
        ctx1.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, tiled.data_ptr())
        ctx1.sync()
        ctx1.set_option(F.OPT_KS_TILED, 0)
        ctx1.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, per_gate.data_ptr())
        ctx1.sync()
    finally:
        ctx1.set_option(F.OPT_KS_TILED, -1)
    assert torch.equal(tiled, per_gate)
    out = host(tiled)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys1.decrypt(out), truth)
    idx = np.array([0, count // 2, count - 1])
    want, failed = keys1.oracle.eval_bootstrap_batch(c1[idx], c2[idx], g[idx], keys1.btkey, keys1.kskey)
    assert failed == 0 and np.array_equal(out[idx], want)


def test_wide_plain_equals_batched(F, ctx1, keys1, cuda_ok):
    """The plain form at N = 2048 (one launch sequence per gate; each lone
    gate's key switch split over many CTAs, 64-bit partial sums reduced mod
    Q per CTA) gives the batched call's words."""
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys1, 3, seed=51)
    d1, d2 = dev(torch, c1), dev(torch, c2)
    dg = torch.from_numpy(g).cuda()
    ob, op = torch.zeros_like(d1), torch.zeros_like(d1)
    ctx1.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 3, ob.data_ptr())
    ctx1.bootstrap_plain_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 3, op.data_ptr())
    ctx1.sync()
    assert torch.equal(ob, op)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys1.decrypt(host(op)), truth)


@pytest.mark.parametrize("count", [20, 60])
def test_wide_rlwe_mult_rgsw_batch(F, ctx1, keys1, cuda_ok, count):
    """One RGSW per product. 20 products (120 product-digit CTAs, at most two
    per SM) take the digit-split kernel; 60 take the one-CTA-per-product kernel
    with the last-digit identity applied to the RGSWs. Both give the oracle's
    words."""
    torch = cuda_ok
    o = keys1.oracle
    Q = keys1.P.Q
    rng = np.random.default_rng(12)
    acc = rng.integers(0, Q, (count, 4096), dtype=np.uint64)
    acc[0] = Q - 1
    acc[1] = 0
    rgsw = rng.integers(0, Q, (count, 6 * 4 * 2048), dtype=np.uint64)
    out = torch.zeros((count, 4096), dtype=torch.int64, device="cuda")
    da, dr = dev(torch, acc), dev(torch, rgsw)
    ctx1.rlwe_mult_rgsw(da.data_ptr(), dr.data_ptr(), out.data_ptr(), count)
    torch.cuda.synchronize()
    assert np.array_equal(host(out), np.stack([o.rlwe_mult_rgsw(acc[i], rgsw[i]) for i in range(count)]))


@pytest.mark.parametrize("pipes,window,compat", [(2, -1, False), (3, 0, False), (2, -1, True)])
def test_wide_remainder_pool(F, ctx1, keys1, pipes, window, compat):
    """13 gates on 2-worker CTAs (7 CTAs of 1 gate, a remainder pool of 6
    that all CTAs share step by step) or 3-worker CTAs (5 of 2, a pool of 3),
    with the step window on and off and in the no-skip issue order: the oracle's
    words, the same as with the pool off, and every gate decrypts."""
    x, y, g, c1, c2 = random_gate_batch(keys1, 13, seed=53)
    flags = F.FLAG_FPGA_COMPAT if compat else 0
    ctx1.set_option(F.OPT_BR_PIPES, pipes)
    ctx1.set_option(F.OPT_BR_WINDOW, window)
    try:
        out = ctx1.eval_bootstrap_batch(c1, c2, g, flags=flags)
        assert ctx1.device_status() == 0
        ctx1.set_option(F.OPT_BR_POOL, 0)
        off = ctx1.eval_bootstrap_batch(c1, c2, g, flags=flags)
    finally:
        ctx1.set_option(F.OPT_BR_POOL, -1)
        ctx1.set_option(F.OPT_BR_PIPES, 0)
        ctx1.set_option(F.OPT_BR_WINDOW, -1)
    want, failed = keys1.oracle.eval_bootstrap_batch(c1, c2, g, keys1.btkey, keys1.kskey, fpga_compat=compat)
    assert failed == 0 or compat
    assert np.array_equal(out, want)
    assert np.array_equal(off, want)
    if not compat:
        truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
        assert np.array_equal(keys1.decrypt(out), truth)


def test_wide_remainder_pool_full_grid(F, ctx1, keys1, cuda_ok):
    """2 x SMs + 37 gates with the default launch: every CTA takes 2 gates of
    its own and the last 37 are shared; all decrypt, a sample on both sides of
    the split equals the oracle, and the NTT-domain accumulators of the
    blind-rotation entry point equal those with the pool off."""
    torch = cuda_ok
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    count = 2 * sms + 37
    x, y, g, c1, c2 = random_gate_batch(keys1, count, seed=57)
    out = ctx1.eval_bootstrap_batch(c1, c2, g)
    assert ctx1.device_status() == 0
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys1.decrypt(out), truth)
    idx = np.array([0, 2 * sms - 1, 2 * sms, 2 * sms + 20, count - 1])
    want, failed = keys1.oracle.eval_bootstrap_batch(c1[idx], c2[idx], g[idx], keys1.btkey, keys1.kskey)
    assert failed == 0
    assert np.array_equal(out[idx], want)
    d1, d2, dg = dev(torch, c1), dev(torch, c2), torch.from_numpy(g).cuda()
    accs = []
    for pool in (-1, 0):
        ctx1.set_option(F.OPT_BR_POOL, pool)
        try:
            acc = torch.zeros((count, 4096), dtype=torch.int64, device="cuda")
            ctx1.blind_rotate_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, acc.data_ptr())
            ctx1.sync()
            accs.append(host(acc))
        finally:
            ctx1.set_option(F.OPT_BR_POOL, -1)
    assert np.array_equal(accs[0], accs[1])
    want_acc, steps = keys1.oracle.blind_rotate(c1[count - 1], c2[count - 1], int(g[count - 1]), keys1.btkey)
    assert np.array_equal(accs[0][count - 1], want_acc)


GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reference_fixture_wide(F, ctx1, keys1, cuda_ok):
    """The 64-bit GPU path word for word against the reference's own outputs
    at N = 2048, Q = 18014398509404161 (ref_bootstrap_p1.npz, made by running
    the reference's RLWE::eval_bootstrap, LWE::LWE_keyswitch and
    LWE::LWE_modswitch, RLWE.cpp:726-786, LWE.cpp:233-269): the truth tables of
    all six gates at n = 32, the key switch on random and edge-word RLWEs, the
    modulus switch on random and edge words, and four gates at n = 630."""
    torch = cuda_ok
    sys.path.insert(0, GOLD)
    from make_ref_fixtures import digest, full_inputs, truth_table_inputs
    from conftest import KeySet
    fx = np.load(os.path.join(GOLD, "ref_bootstrap_p1.npz"))
    small = KeySet(F, 1, n=int(fx["n_small"]))
    x, y, g, c1, c2 = truth_table_inputs(small)
    assert digest(c1, c2) == fx["inputs_sha256"].item().decode()
    with F.Context(small.P, 0) as ctx:
        ctx.upload_bootstrap_key(small.btkey)
        ctx.upload_keyswitch_key(small.kskey)
        out = ctx.eval_bootstrap_batch(c1, c2, g)
        assert np.array_equal(out, fx["out"].astype(np.uint64))
        rl = fx["ks_in"]
        dr = dev(torch, rl)
        ks = torch.zeros((rl.shape[0], small.P.n + 1), dtype=torch.int64, device="cuda")
        ctx.lwe_keyswitch_async(dr.data_ptr(), rl.shape[0], ks.data_ptr())
        ctx.sync()
        assert np.array_equal(host(ks), fx["ks_out"])
        lw = fx["ms_in"]
        dl = dev(torch, lw)
        ms = torch.zeros_like(dl)
        ctx.lwe_modswitch_async(dl.data_ptr(), lw.shape[0], ms.data_ptr())
        ctx.sync()
        assert np.array_equal(host(ms), fx["ms_out"])
    fx_, fy, fg, f1, f2 = full_inputs(keys1)
    assert digest(f1, f2) == fx["full_inputs_sha256"].item().decode()
    fout = ctx1.eval_bootstrap_batch(f1, f2, fg)
    assert np.array_equal(fout, fx["full_out"].astype(np.uint64))


def test_wide_verify_keys(F, ctx1, keys1, cuda_ok):
    """Read-back verification at N = 2048 (keys held as Shoup pairs made on
    the GPU): the resident bootstrap and substitute keys compare equal to the
    keys they were uploaded from, and a copy with one word changed does not."""
    assert ctx1.verify_bootstrap_key(keys1.btkey)
    keys1.btkey[11] ^= 1   # in place (the key is 11.4 GB), restored below
    try:
        assert not ctx1.verify_bootstrap_key(keys1.btkey)
    finally:
        keys1.btkey[11] ^= 1
    assert ctx1.verify_bootstrap_key(keys1.btkey)
    ctx1.upload_subs_key(keys1.subs)
    assert ctx1.verify_subs_key(keys1.subs)
    bad_subs = keys1.subs.copy()
    bad_subs[-3] ^= 1
    assert not ctx1.verify_subs_key(bad_subs)
