"""The latency form of the 32-bit blind rotation (one CTA per ciphertext,
accumulator in shared memory, keys prefetched by bulk asynchronous copies),
which the library takes up to one gate per SM, against the pipelined kernel on
the same inputs and against the oracle. Both run the reference's
RLWE::eval_bootstrap accumulate loop (RLWE.cpp:733-767) with the same
arithmetic, so every word must match (integer arithmetic, tolerance 0)."""
import numpy as np
import pytest

from conftest import KeySet, random_gate_batch, x1_gate_batch

pytestmark = pytest.mark.gpu


def _both_forms(F, ctx, run):
    """run() with the pipelines (FHEACC_OPT_BR_SOLO 0) and with the latency
    form for up to two gates per SM (2)."""
    try:
        ctx.set_option(F.OPT_BR_SOLO, 0)
        pipes = run()
        ctx.set_option(F.OPT_BR_SOLO, 2)
        solo = run()
    finally:
        ctx.set_option(F.OPT_BR_SOLO, -1)
    return pipes, solo


@pytest.mark.parametrize("count", [1, 40, 152, 300])
@pytest.mark.parametrize("order", ["cpu", "fpga_compat", "fpga_x1"])
def test_latency_form_equals_pipelines(F, ctx0, keys0, cuda_ok, count, order):
    if order == "fpga_x1":
        x, y, g, c1, c2, _ = x1_gate_batch(keys0, count, seed=500 + count)
    else:
        x, y, g, c1, c2 = random_gate_batch(keys0, count, seed=400 + count)
    flags = {"cpu": 0, "fpga_compat": F.FLAG_FPGA_COMPAT, "fpga_x1": F.FLAG_FPGA_X1}[order]
    pipes, solo = _both_forms(F, ctx0, lambda: ctx0.eval_bootstrap_batch(c1, c2, g, flags=flags))
    assert np.array_equal(solo, pipes)
    assert ctx0.device_status() == 0
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(solo), truth)


def test_latency_form_accumulators(F, ctx0, keys0, cuda_ok):
    """The canonical NTT-domain accumulators (fheacc_blind_rotate_async), one
    ciphertext per CTA, equal the pipelines' and the oracle's."""
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys0, 5, seed=451)
    d1 = torch.from_numpy(c1.view(np.int64)).cuda()
    d2 = torch.from_numpy(c2.view(np.int64)).cuda()
    dg = torch.from_numpy(g).cuda()

    def run():
        acc = torch.zeros((5, 2048), dtype=torch.int64, device="cuda")
        ctx0.blind_rotate_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 5, acc.data_ptr())
        torch.cuda.synchronize()
        return acc.cpu().numpy().view(np.uint64)

    pipes, solo = _both_forms(F, ctx0, run)
    assert np.array_equal(solo, pipes)
    for k in range(5):
        want, steps = keys0.oracle.blind_rotate(c1[k], c2[k], int(g[k]), keys0.btkey)
        assert steps > 900
        assert np.array_equal(solo[k], want), "gate %d" % k


@pytest.fixture(scope="module")
def keys2(F):
    """Preset 2 (N = 1024, Q < 2^27, BG = 2^9 x 3) with n = 64: the latency
    form's digitG = 3 instantiation and single-copy digit tables."""
    return KeySet(F, 2, n=64)


def test_latency_form_bg9_against_oracle(F, keys2, cuda_ok):
    ctx = F.Context(keys2.P, 0)
    try:
        ctx.upload_bootstrap_key(keys2.btkey)
        ctx.upload_keyswitch_key(keys2.kskey)
        x, y, g, c1, c2 = random_gate_batch(keys2, 9, seed=461)
        pipes, solo = _both_forms(F, ctx, lambda: ctx.eval_bootstrap_batch(c1, c2, g))
        assert np.array_equal(solo, pipes)
        want, failed = keys2.oracle.eval_bootstrap_batch(c1, c2, g, keys2.btkey, keys2.kskey)
        assert failed == 0
        assert np.array_equal(solo, want)
        assert ctx.device_status() == 0
    finally:
        ctx.close()


def test_empty_batches_launch_nothing(F, ctx0, cuda_ok):
    """count = 0 through every bootstrap entry point: FHEACC_OK, no kernel
    launched, no output touched (the reference's x-width calls reject a
    wrong width; an any-count ABI takes zero as a no-op)."""
    torch = cuda_ok
    L = F.lib()
    d = torch.full((4, 501), -1, dtype=torch.int64, device="cuda")
    dg = torch.zeros(4, dtype=torch.int32, device="cuda")
    before = ctx0.kernel_launches() if hasattr(ctx0, "kernel_launches") else None
    ctx0.bootstrap_async(d.data_ptr(), d.data_ptr(), dg.data_ptr(), 0, d.data_ptr())
    ctx0.bootstrap_plain_async(d.data_ptr(), d.data_ptr(), dg.data_ptr(), 0, d.data_ptr())
    ctx0.blind_rotate_async(d.data_ptr(), d.data_ptr(), dg.data_ptr(), 0, d.data_ptr())
    assert L.fheacc_bootstrap_noalloc(ctx0.handle, d.data_ptr(), d.data_ptr(), dg.data_ptr(), 0, d.data_ptr(), 0,
                                      None) == F.OK
    assert L.fheacc_bootstrap(ctx0.handle, None, None, None, 0, None, 0) == F.OK
    ctx0.sync()
    if before is not None:
        assert ctx0.kernel_launches() == before
    assert bool((d == -1).all())
