"""Bounded device waits that run out. The blind-rotation workers of a CTA
wait for each other when two of them hold consecutive steps of one
ciphertext; every such wait is bounded, and a wait that gives up flags the
launch's results invalid instead of hanging the GPU. FHEACC_OPT_DEBUG_WAIT_LIMIT
shrinks the bounds to zero polls, so that on a one-gate batch spread over
several workers of one CTA the second worker's first wait expires: the kernel
returns, fheacc_device_status reports FHEACC_STATUS_WAIT_LIMIT, fheacc_sync
returns FHEACC_EIO, and the context works again once the limit is restored.
Nothing here faults or hangs a GPU: the waits end by their own bound."""
import ctypes

import numpy as np
import pytest

from conftest import random_gate_batch

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64) if a.dtype == np.uint64 else a).cuda()


def _expiry(F, ctx, keys, torch, workers, seed):
    L = F.lib()
    x, y, g, c1, c2 = random_gate_batch(keys, 1, seed=seed)
    d1, d2, dg = _dev(torch, c1), _dev(torch, c2), torch.from_numpy(g).cuda()
    out = torch.zeros_like(d1)
    assert ctx.device_status() == 0
    ctx.set_option(F.OPT_BR_PIPES, workers)
    ctx.set_option(F.OPT_DEBUG_WAIT_LIMIT, 0)
    try:
        # the status word, read directly
        ctx.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 1, out.data_ptr())
        torch.cuda.synchronize()
        bits = ctypes.c_uint32()
        rc = L.fheacc_device_status(ctx.handle, ctypes.byref(bits))
        assert rc == F.EIO
        assert bits.value & F.STATUS_WAIT_LIMIT
        # fheacc_sync reports the same failure
        ctx.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 1, out.data_ptr())
        assert L.fheacc_sync(ctx.handle, 60000) == F.EIO
        assert b"bounded wait" in L.fheacc_last_error(ctx.handle)
    finally:
        ctx.set_option(F.OPT_DEBUG_WAIT_LIMIT, -1)
        ctx.set_option(F.OPT_BR_PIPES, 0)
    # built-in limits again: the same launch shape gives correct results
    ctx.set_option(F.OPT_BR_PIPES, workers)
    try:
        ctx.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 1, out.data_ptr())
        ctx.sync()
    finally:
        ctx.set_option(F.OPT_BR_PIPES, 0)
    assert ctx.device_status() == 0
    truth = np.array([F.gate_truth(int(g[0]), x[0], y[0])], dtype=np.uint8)
    assert np.array_equal(keys.decrypt(out.cpu().numpy().view(np.uint64)), truth)


def test_wait_limit_expires_32bit(F, ctx0, keys0, cuda_ok):
    """Three pipelines share one CTA's one-gate group: the second and third
    pipeline each claim a later step of the gate and wait for the first."""
    _expiry(F, ctx0, keys0, cuda_ok, workers=3, seed=4401)


def test_wait_limit_expires_64bit(F, ctx1, keys1, cuda_ok):
    """Two workers share one CTA's one-gate group (N = 2048, 64-bit words)."""
    _expiry(F, ctx1, keys1, cuda_ok, workers=2, seed=4402)


def test_debug_wait_limit_rejects_negative(F, ctx0, cuda_ok):
    L = F.lib()
    assert L.fheacc_set_option(ctx0.handle, F.OPT_DEBUG_WAIT_LIMIT, -2) == F.EINVAL
