"""fheacc_bootstrap_noalloc: gate bootstrapping for callers that may not
allocate device memory while they run (a serving loop that must not let
cudaFree synchronise the shared GPU, a process under a fixed memory
reservation). Its scratch is a fixed array inside the library, so it takes at
most FHEACC_NOALLOC_MAX_GATES gates per call. It must give exactly the words
of the allocating entry point, fheacc_bootstrap_async, call after call.

Collected last on purpose (tests/ runs alphabetically): if it fails, a run
that stops at the first failure has already run every other test."""
import numpy as np
import pytest

from conftest import random_gate_batch

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64) if a.dtype == np.uint64 else a).cuda()


def test_noalloc_equals_allocating_entry_point_two_calls(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    L = F.lib()
    batches = [random_gate_batch(keys0, 40, seed=909), random_gate_batch(keys0, F.NOALLOC_MAX_GATES, seed=910)]
    for x, y, g, c1, c2 in batches:   # two calls in a row, different inputs
        d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
        count = c1.shape[0]
        want = torch.zeros_like(d1)
        ctx0.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count, want.data_ptr())
        got = torch.full_like(d1, -1)
        rc = L.fheacc_bootstrap_noalloc(ctx0.handle, d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), count,
                                        got.data_ptr(), 0, None)
        assert rc == F.OK, L.fheacc_last_error(ctx0.handle)
        torch.cuda.synchronize()
        assert torch.equal(got, want)   # bit-exact, the tolerance of every parity test here
        truth = np.array([F.gate_truth(int(a), b, c) for a, b, c in zip(g, x, y)], dtype=np.uint8)
        assert np.array_equal(keys0.decrypt(got.cpu().numpy().view(np.uint64)), truth)


def test_noalloc_rejects_more_than_max(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    L = F.lib()
    n = F.NOALLOC_MAX_GATES + 1
    x, y, g, c1, c2 = random_gate_batch(keys0, n, seed=911)
    d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
    out = torch.zeros_like(d1)
    rc = L.fheacc_bootstrap_noalloc(ctx0.handle, d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), n, out.data_ptr(),
                                    0, None)
    assert rc == F.EINVAL
    assert b"FHEACC_NOALLOC_MAX_GATES" in L.fheacc_last_error(ctx0.handle)
    torch.cuda.synchronize()
    assert int(out.abs().sum()) == 0   # nothing was launched
