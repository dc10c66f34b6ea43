"""Batched bootstraps of several parameter sets in one CUDA-graph launch, and
the launch-shape autotuner: outputs equal the one-call-per-batch path
(fheacc_bootstrap_async) word for word, and decrypt to the gate values."""
import numpy as np
import pytest

from conftest import KeySet, random_gate_batch

pytestmark = pytest.mark.gpu


def dev(torch, a, dtype=np.uint64):
    a = np.ascontiguousarray(a, dtype=dtype)
    return torch.from_numpy(a.view(np.int64) if dtype == np.uint64 else a).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


class SmallKeys(KeySet):
    """The bench parameter set with n = 64 (same N, Q and gadget): a second
    32-bit context with small keys."""

    def __init__(self, F):
        P = F.params_preset(0)
        P.n = 64
        F.derive(P)
        self.P = P
        self.lwe_sk = F.LWE_secretkey(P, 21)
        self.rlwe_sk = F.RLWE_secretkey(P, 22)
        self.btkey = F.bootstrap_key(P, 23, self.lwe_sk, self.rlwe_sk)
        self.kskey = F.keyswitch_key(P, 24, self.rlwe_sk, self.lwe_sk)
        self._subs = None
        self.F = F


@pytest.fixture(scope="module")
def small(F, cuda_ok):
    ks = SmallKeys(F)
    ctx = F.Context(ks.P, 0)
    ctx.upload_bootstrap_key(ks.btkey)
    ctx.upload_keyswitch_key(ks.kskey)
    yield ks, ctx
    ctx.close()


def batch_on_device(torch, ks, count, seed):
    x, y, g, c1, c2 = random_gate_batch(ks, count, seed)
    truth = np.array([ks.F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    d = dict(c1=dev(torch, c1), c2=dev(torch, c2), g=dev(torch, g, np.int32),
             out=torch.zeros((count, ks.P.n + 1), dtype=torch.int64, device="cuda"))
    return d, truth


def direct(torch, ctx, d, count):
    out = torch.zeros_like(d["out"])
    ctx.bootstrap_async(d["c1"].data_ptr(), d["c2"].data_ptr(), d["g"].data_ptr(), count, out.data_ptr(), 0, 0)
    torch.cuda.synchronize()
    return host(out)


@pytest.mark.parametrize("concurrent", [False, True])
def test_graph_two_parameter_sets(F, ctx0, keys0, small, cuda_ok, concurrent):
    torch = cuda_ok
    ks, ctxs = small
    jobs = [(ctx0, keys0, 37, 1), (ctxs, ks, 200, 2), (ctx0, keys0, 300, 3), (ctxs, ks, 5, 4)]
    data = [batch_on_device(torch, k, n, s) for _, k, n, s in jobs]
    g = F.Graph(concurrent)
    for (ctx, k, n, s), (d, _) in zip(jobs, data):
        g.add(ctx, d["c1"].data_ptr(), d["c2"].data_ptr(), d["g"].data_ptr(), n, d["out"].data_ptr())
    assert g.batches == 4
    for _ in range(2):   # capture at the first launch, replay at the second
        for d, _ in data:
            d["out"].zero_()
        g.launch()
        torch.cuda.synchronize()
        for (ctx, k, n, s), (d, truth) in zip(jobs, data):
            o = host(d["out"])
            assert np.array_equal(o, direct(torch, ctx, d, n))
            assert np.array_equal(k.decrypt(o), truth)
    g.close()


def test_graph_narrow_and_wide(F, ctx0, keys0, ctx1, keys1, cuda_ok):
    """One graph launch mixing N = 1024 (32-bit) and N = 2048 (64-bit) gates."""
    torch = cuda_ok
    jobs = [(ctx0, keys0, 64, 5), (ctx1, keys1, 6, 6)]
    data = [batch_on_device(torch, k, n, s) for _, k, n, s in jobs]
    g = F.Graph(concurrent=True)
    for (ctx, k, n, s), (d, _) in zip(jobs, data):
        g.add(ctx, d["c1"].data_ptr(), d["c2"].data_ptr(), d["g"].data_ptr(), n, d["out"].data_ptr())
    g.launch()
    torch.cuda.synchronize()
    for (ctx, k, n, s), (d, truth) in zip(jobs, data):
        o = host(d["out"])
        assert np.array_equal(o, direct(torch, ctx, d, n))
        assert np.array_equal(k.decrypt(o), truth)
    g.close()


def test_graph_errors(F, ctx0, small, cuda_ok):
    g = F.Graph()
    g.launch()   # empty graph: nothing to do
    with pytest.raises(F.FheaccError):
        g.add(ctx0, 0, 0, 0, 3, 0)
    g.close()


def test_autotune_keeps_results(F, small, cuda_ok):
    torch = cuda_ok
    ks, ctx = small
    d, truth = batch_on_device(torch, ks, 300, 7)
    before = direct(torch, ctx, d, 300)
    trials = ctx.autotune(300)
    assert len(trials) >= 4 and all(t["ms"] > 0 for t in trials)
    after = direct(torch, ctx, d, 300)
    assert np.array_equal(before, after) and np.array_equal(ks.decrypt(after), truth)
    assert {t["pipes"] for t in trials} >= {1, 3}
    # every tried shape gives the same words
    for t in trials:
        ctx.set_option(F.OPT_BR_REGS_FOR_3, t["regs_for_3"])
        ctx.set_option(F.OPT_BR_CTAS_PER_SM, t["ctas_per_sm"])
        ctx.set_option(F.OPT_BR_GROUP, t["group"])
        ctx.set_option(F.OPT_BR_WINDOW, t["window"])
        ctx.set_option(F.OPT_BR_PIPES, t["pipes"])
        assert np.array_equal(direct(torch, ctx, d, 300), before)
    ctx.set_option(F.OPT_BR_REGS_FOR_3, -1)   # back to the defaults
    ctx.set_option(F.OPT_BR_WINDOW, -1)
    ctx.set_option(F.OPT_BR_PIPES, 0)
    for o in (F.OPT_BR_CTAS_PER_SM, F.OPT_BR_GROUP):
        ctx.set_option(o, 0)
