"""fheacc_bootstrap_noalloc: gate bootstrapping for callers that may not
allocate device memory while they run (a serving loop that must not let
cudaFree synchronise the shared GPU, a process under a fixed memory
reservation). Its scratch is a fixed array inside the library, so it takes at
most FHEACC_NOALLOC_MAX_GATES gates per call. It must give exactly the words
of the allocating entry point, fheacc_bootstrap_async, call after call.

The no-alloc calls run on a context of their own that has never run the
allocating path, so a hidden growth of the context's scratch would show in
fheacc_device_bytes; the allocating path runs on the shared session context.

Collected last on purpose (tests/ runs alphabetically): if it fails, a run
that stops at the first failure has already run every other test."""
import numpy as np
import pytest

from conftest import random_gate_batch

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64) if a.dtype == np.uint64 else a).cuda()


@pytest.fixture(scope="module")
def noalloc_ctx(F, keys0, cuda_ok):
    ctx = F.Context(keys0.P, 0)
    ctx.upload_bootstrap_key(keys0.btkey)
    ctx.upload_keyswitch_key(keys0.kskey)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("flags", [0, 1], ids=["cpu_order", "fpga_compat"])
def test_noalloc_equals_allocating_entry_point_two_calls(F, noalloc_ctx, ctx0, keys0, cuda_ok, flags):
    torch = cuda_ok
    L = F.lib()
    assert flags in (0, F.FLAG_FPGA_COMPAT)
    batches = [random_gate_batch(keys0, 40, seed=909 + 2 * flags),
               random_gate_batch(keys0, F.NOALLOC_MAX_GATES, seed=910 + 2 * flags)]
    for x, y, g, c1, c2 in batches:   # two calls in a row, different inputs
        d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
        count = c1.shape[0]
        got = torch.full_like(d1, -1)
        held = noalloc_ctx.device_bytes()
        rc = L.fheacc_bootstrap_noalloc(noalloc_ctx.handle, d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count,
                                        got.data_ptr(), flags, None)
        assert rc == F.OK, L.fheacc_last_error(noalloc_ctx.handle)
        torch.cuda.synchronize()
        assert noalloc_ctx.device_bytes() == held   # the call grew no scratch of the context
        want = torch.zeros_like(d1)
        ctx0.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, want.data_ptr(), flags=flags)
        torch.cuda.synchronize()
        assert torch.equal(got, want)   # bit-exact, the tolerance of every parity test here
        truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
        assert np.array_equal(keys0.decrypt(got.cpu().numpy().view(np.uint64)), truth)


def test_noalloc_profile_flag_records_times(F, noalloc_ctx, keys0, cuda_ok):
    torch = cuda_ok
    L = F.lib()
    x, y, g, c1, c2 = random_gate_batch(keys0, 8, seed=913)
    d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
    out = torch.zeros_like(d1)
    rc = L.fheacc_bootstrap_noalloc(noalloc_ctx.handle, d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 8,
                                    out.data_ptr(), F.FLAG_PROFILE, None)
    assert rc == F.OK, L.fheacc_last_error(noalloc_ctx.handle)
    br_ms, ks_ms = noalloc_ctx.kernel_times()
    assert br_ms > 0 and ks_ms > 0
    truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
    assert np.array_equal(keys0.decrypt(out.cpu().numpy().view(np.uint64)), truth)


def test_noalloc_rejects_more_than_max(F, noalloc_ctx, keys0, cuda_ok):
    torch = cuda_ok
    L = F.lib()
    n = F.NOALLOC_MAX_GATES + 1
    x, y, g, c1, c2 = random_gate_batch(keys0, n, seed=911)
    d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
    out = torch.zeros_like(d1)
    rc = L.fheacc_bootstrap_noalloc(noalloc_ctx.handle, d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), n,
                                    out.data_ptr(), 0, None)
    assert rc == F.EINVAL
    assert b"FHEACC_NOALLOC_MAX_GATES" in L.fheacc_last_error(noalloc_ctx.handle)
    torch.cuda.synchronize()
    assert int(out.abs().sum()) == 0   # nothing was launched
