"""Gate bootstrapping on the GPU, end to end, against the oracle (bit-exact)
and by decryption (the truth tables of test::bootstrapping, test.cpp:496-625).
"""
import numpy as np
import pytest

from conftest import random_gate_batch, x1_gate_batch

pytestmark = pytest.mark.gpu


def test_truth_tables_all_gates(F, ctx0, keys0):
    """Every gate on every input pair, as test::bootstrapping does."""
    xs, ys, gs = [], [], []
    for g in range(6):
        for a in (0, 1):
            for b in (0, 1):
                xs.append(a); ys.append(b); gs.append(g)
    x = np.array(xs, dtype=np.uint8); y = np.array(ys, dtype=np.uint8); g = np.array(gs, dtype=np.int32)
    c = keys0.encrypt(np.concatenate([x, y]), seed=77)
    c1, c2 = c[:24], c[24:]
    out = ctx0.eval_bootstrap_batch(c1, c2, g)
    want, failed = keys0.oracle.eval_bootstrap_batch(c1, c2, g, keys0.btkey, keys0.kskey)
    assert failed == 0
    assert np.array_equal(out, want)
    dec = keys0.decrypt(out)
    truth = np.array([F.gate_truth(int(gg), a, b) for gg, a, b in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(dec, truth)


@pytest.mark.parametrize("count", [1, 33])
def test_batch_bitexact(F, ctx0, keys0, count):
    x, y, g, c1, c2 = random_gate_batch(keys0, count, seed=100 + count)
    out = ctx0.eval_bootstrap_batch(c1, c2, g)
    want, failed = keys0.oracle.eval_bootstrap_batch(c1, c2, g, keys0.btkey, keys0.kskey)
    assert failed == 0
    assert np.array_equal(out, want)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)


def test_plain_equals_batched(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys0, 5, seed=7)
    d1 = torch.from_numpy(c1.view(np.int64)).cuda()
    d2 = torch.from_numpy(c2.view(np.int64)).cuda()
    dg = torch.from_numpy(g).cuda()
    ob = torch.zeros_like(d1)
    op = torch.zeros_like(d1)
    ctx0.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 5, ob.data_ptr())
    ctx0.bootstrap_plain_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 5, op.data_ptr())
    ctx0.sync()
    assert torch.equal(ob, op)
    assert np.array_equal(ob.cpu().numpy().view(np.uint64), ctx0.eval_bootstrap_batch(c1, c2, g))


@pytest.mark.parametrize("pipes", [0, 1, 2, 3])
def test_fpga_compat_mode(F, ctx0, keys0, pipes):
    """The no-skip issue order of fpga_eval_bootstrap_x4..x16
    (myfpga.cpp:1200-1210) against the oracle run the same way, with every
    number of pipelines per CTA (their shared cursor then issues every step)."""
    x, y, g, c1, c2 = random_gate_batch(keys0, 7, seed=3)
    ctx0.set_option(F.OPT_BR_PIPES, pipes)
    try:
        out = ctx0.eval_bootstrap_batch(c1, c2, g, flags=F.FLAG_FPGA_COMPAT)
    finally:
        ctx0.set_option(F.OPT_BR_PIPES, 0)
    want, failed = keys0.oracle.eval_bootstrap_batch(c1, c2, g, keys0.btkey, keys0.kskey, fpga_compat=True)
    assert np.array_equal(out, want)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)


@pytest.mark.parametrize("pipes", [0, 1, 3])
def test_fpga_x1_mode(F, ctx0, keys0, pipes):
    """The issue order of fpga_eval_bootstrap_x1 (myfpga.cpp:1037-1046: the
    first step always, with residue 0's key when its residue is 0) against the
    oracle run the same way; gates with a non-zero first residue equal the CPU
    path's words."""
    x, y, g, c1, c2, zero = x1_gate_batch(keys0, 6, seed=61)
    ctx0.set_option(F.OPT_BR_PIPES, pipes)
    try:
        out = ctx0.eval_bootstrap_batch(c1, c2, g, flags=F.FLAG_FPGA_X1)
        cpu_order = ctx0.eval_bootstrap_batch(c1, c2, g)
    finally:
        ctx0.set_option(F.OPT_BR_PIPES, 0)
    want, failed = keys0.oracle.eval_bootstrap_batch(c1, c2, g, keys0.btkey, keys0.kskey, fpga_compat=2)
    assert failed == 0
    assert np.array_equal(out, want)
    assert np.array_equal(out[~zero], cpu_order[~zero])
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)


def test_gpu_fixed_width_calls(F, ctx0, keys0):
    """The fixed-width counterparts of fpga_eval_bootstrap_x4/x8/x12/x16:
    x16 takes exactly 10 gates (myfpga.cpp:1540-1544), other sizes give
    rc = -1 and no result."""
    x, y, g, c1, c2 = random_gate_batch(keys0, 12, seed=71)
    for width, call in ((4, ctx0.gpu_eval_bootstrap_x4), (8, ctx0.gpu_eval_bootstrap_x8),
                        (12, ctx0.gpu_eval_bootstrap_x12), (10, ctx0.gpu_eval_bootstrap_x16)):
        out, rc = call(list(c1[:width]), list(c2[:width]), list(g[:width]))
        assert rc == 0
        assert np.array_equal(np.array(out), ctx0.eval_bootstrap_batch(c1[:width], c2[:width], g[:width]))
        bad, rc = call(list(c1[:width - 1]), list(c2[:width - 1]), list(g[:width - 1]))
        assert bad is None and rc == -1
    out, rc = ctx0.gpu_eval_bootstrap_x16(list(c1[:12]), list(c2[:12]), list(g[:12]))
    assert out is None and rc == -1


@pytest.mark.parametrize("count", [40, 333, 1100, 2600])
def test_tiled_keyswitch_equals_per_gate(F, ctx0, keys0, cuda_ok, count):
    """The tiled LWE key switch (gate blocks sharing each key row group through
    shared memory; batches from 1024 gates take it by default) against the
    one-CTA-per-gate kernel on the same blind-rotation outputs: forced on small
    batches, with a partial last gate block (40, 333: 16 gates per block) and
    two and five gates per warp (1100, 2600); the first gates also against the
    oracle."""
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys0, count, seed=81 + count)
    d1 = torch.from_numpy(c1.view(np.int64)).cuda()
    d2 = torch.from_numpy(c2.view(np.int64)).cuda()
    dg = torch.from_numpy(g).cuda()
    tiled, per_gate = torch.zeros_like(d1), torch.zeros_like(d1)
    try:
        ctx0.set_option(F.OPT_KS_TILED, 1)
        ctx0.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, tiled.data_ptr())
        ctx0.sync()
        ctx0.set_option(F.OPT_KS_TILED, 0)
        ctx0.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, per_gate.data_ptr())
        ctx0.sync()
    finally:
        ctx0.set_option(F.OPT_KS_TILED, -1)
    assert torch.equal(tiled, per_gate)
    out = tiled.cpu().numpy().view(np.uint64)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)
    k = 6
    want, failed = keys0.oracle.eval_bootstrap_batch(c1[:k], c2[:k], g[:k], keys0.btkey, keys0.kskey)
    assert failed == 0 and np.array_equal(out[:k], want)


def test_errors(F, ctx0, keys0):
    x, y, g, c1, c2 = random_gate_batch(keys0, 2, seed=5)
    with pytest.raises(F.FheaccError) as e:
        ctx0.eval_bootstrap_batch(c1, c1, g)          # c1 == c2 (RLWE.cpp:727-730)
    assert e.value.code == F.EINVAL
    with pytest.raises(F.FheaccError):
        ctx0.eval_bootstrap_batch(c1, c2, [7, 0])     # bad gate code
    assert ctx0.eval_bootstrap_batch(c1[:0], c2[:0], np.zeros(0, dtype=np.int32)).shape == (0, keys0.P.n + 1)
    res, rc = ctx0.gpu_eval_bootstrap_x4(list(c1), list(c2), list(g))   # wrong width
    assert res is None and rc == -1


def test_kernel_launch_count(F, ctx0, keys0):
    """The context counts its kernel launches: a batched bootstrap launches a
    fixed, small number of kernels (blind rotation, key switch), the same for
    the same call."""
    x, y, g, c1, c2 = random_gate_batch(keys0, 40, seed=61)
    counts = []
    for _ in range(2):
        n0 = ctx0.kernel_launches()
        ctx0.eval_bootstrap_batch(c1, c2, g)
        counts.append(ctx0.kernel_launches() - n0)
    assert counts[0] == counts[1] and 2 <= counts[0] <= 4


def test_fixed_width_wrappers(F, ctx0, keys0):
    x, y, g, c1, c2 = random_gate_batch(keys0, 4, seed=44)
    res, rc = ctx0.gpu_eval_bootstrap_x4(list(c1), list(c2), list(g))
    assert rc == 0
    assert np.array_equal(np.array(res), ctx0.eval_bootstrap_batch(c1, c2, g))
    one, rc = ctx0.gpu_eval_bootstrap_x1(c1[0], c2[0], int(g[0]))
    assert rc == 0 and np.array_equal(one, res[0])


def test_reference_fixture(F, ctx0, keys0):
    """GPU outputs equal the words the reference's own eval_bootstrap produced
    for the same seeded keys and inputs (tests/golden/make_ref_fixtures.py)."""
    import os
    import sys
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, gold)
    from make_ref_fixtures import digest, truth_table_inputs
    fx = np.load(os.path.join(gold, "ref_bootstrap_p0.npz"))
    x, y, g, c1, c2 = truth_table_inputs(keys0)
    assert digest(c1, c2) == fx["inputs_sha256"].item().decode()
    out = ctx0.eval_bootstrap_batch(c1, c2, g)
    assert np.array_equal(out, fx["out"].astype(np.uint64))


@pytest.mark.parametrize("count,group", [(12007, 0), (1021, 3), (2, 0)])
def test_large_and_ragged_batches(F, ctx0, keys0, count, group):
    """Batches that take several chunks per CTA (12007 gates: more than the
    grid holds in one group), uneven groups under a small cap (1021 gates,
    at most 3 per CTA) and a batch smaller than one group per CTA: every
    gate decrypts, and a sample (first, last and spread) equals the oracle."""
    x, y, g, c1, c2 = random_gate_batch(keys0, count, seed=200 + count)
    ctx0.set_option(F.OPT_BR_GROUP, group)
    try:
        out = ctx0.eval_bootstrap_batch(c1, c2, g)
    finally:
        ctx0.set_option(F.OPT_BR_GROUP, 0)
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out), truth)
    idx = np.unique(np.concatenate([[0, count - 1], np.linspace(0, count - 1, 14).astype(int)]))
    want, failed = keys0.oracle.eval_bootstrap_batch(c1[idx], c2[idx], g[idx], keys0.btkey, keys0.kskey)
    assert failed == 0
    assert np.array_equal(out[idx], want)


def test_verify_keys(F, ctx0, keys0):
    """Read-back verification (dma_read_compare_bootstrap_key,
    myfpga.cpp:772-851): the resident bootstrap key compares equal to the key
    it was uploaded from; a copy with one word changed, early or late in the
    device order, does not; a context without a key reports it."""
    assert ctx0.verify_bootstrap_key(keys0.btkey)
    for at in (5, keys0.btkey.size - 17):
        keys0.btkey[at] ^= 1   # in place, restored below
        try:
            assert not ctx0.verify_bootstrap_key(keys0.btkey)
        finally:
            keys0.btkey[at] ^= 1
    assert ctx0.verify_bootstrap_key(keys0.btkey)
    with F.Context(keys0.P, 0) as fresh:
        with pytest.raises(F.FheaccError) as e:
            fresh.verify_bootstrap_key(keys0.btkey)
        assert e.value.code == F.ENOKEY
