"""The continuous-batching server: PSI-style equality queries (XNOR + AND-tree
circuits of gate bootstraps) give the same output words alone and mixed with
concurrent traffic, and decrypt to the right equality bits."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_query(F, ks, items, match_at, seed):
    """Client item + server items (one equal to the client's at match_at)."""
    rng = np.random.default_rng(seed)
    client = int(rng.integers(0, 1 << 32))
    server = [int(v) for v in rng.integers(0, 1 << 32, items)]
    if match_at is not None:
        server[match_at] = client
    bits = [(client >> b) & 1 for b in range(32)]
    for v in server:
        bits += [(v >> b) & 1 for b in range(32)]
    ct = ks.encrypt(np.array(bits, dtype=np.uint8), seed=10_000 + seed)
    want = np.array([int(v == client) for v in server], dtype=np.uint8)
    return ct, want


def wait_all(srv, ids, timeout_s=120):
    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < timeout_s:
        for rid, status, q_ms, lat_ms, out in srv.poll(timeout_ms=200):
            got[rid] = (status, out, lat_ms)
    assert len(got) == len(ids), "requests did not complete"
    return got


def test_server_same_alone_and_in_mix(F, ctx0, keys0):
    srv = F.Server(ctx0, max_batch=2048, pool_ciphertexts=1 << 16)
    try:
        circ = F.psi_equality_circuit(3)
        ct, want = make_query(F, keys0, 3, match_at=1, seed=1)
        rid, _ = srv.submit(ct, *circ)
        alone = wait_all(srv, [rid])[rid]
        assert alone[0] == F.OK
        assert np.array_equal(keys0.decrypt(alone[1]), want)

        # the same request again, submitted from two threads among 12 others
        others = [make_query(F, keys0, k, match_at=(0 if k % 2 else None), seed=100 + k) for k in range(1, 13)]
        ids, wants = [], {}
        lock = threading.Lock()

        def feed(chunk):
            for ct_o, want_o in chunk:
                r, _ = srv.submit(ct_o, *F.psi_equality_circuit(len(want_o)))
                with lock:
                    ids.append(r)
                    wants[r] = want_o
                time.sleep(0.002)

        th = [threading.Thread(target=feed, args=(others[i::2],)) for i in range(2)]
        for t in th:
            t.start()
        rid2, _ = srv.submit(ct, *circ)
        for t in th:
            t.join()
        got = wait_all(srv, ids + [rid2])
        assert got[rid2][0] == F.OK
        assert np.array_equal(got[rid2][1], alone[1]), "result differs when mixed with other requests"
        for r in ids:
            assert got[r][0] == F.OK
            assert np.array_equal(keys0.decrypt(got[r][1]), wants[r])
        st = srv.stats()
        assert st["gates"] == 63 * (3 + 3 + sum(range(1, 13)))
        assert st["rounds"] < st["gates"]          # gates of different requests shared launches
        assert st["free_slots"] == (1 << 16)       # every slot released
    finally:
        srv.close()


def test_server_admission_waits_for_room(F, ctx0, keys0):
    """A pool that fits one request at a time still completes all of them,
    in arrival order, each result correct (admission by free device memory)."""
    circ = F.psi_equality_circuit(2)
    need = 32 * 3 + len(circ[0])
    srv = F.Server(ctx0, max_batch=512, pool_ciphertexts=need)
    try:
        qs = [make_query(F, keys0, 2, match_at=i % 2, seed=200 + i) for i in range(4)]
        ids = [srv.submit(ct, *circ)[0] for ct, _ in qs]
        got = wait_all(srv, ids)
        for rid, (_, want) in zip(ids, qs):
            assert got[rid][0] == F.OK
            assert np.array_equal(keys0.decrypt(got[rid][1]), want)
        lat = [got[r][2] for r in ids]
        assert lat == sorted(lat)   # served one after another
    finally:
        srv.close()


def test_server_rejects_bad_circuits(F, ctx0, keys0):
    srv = F.Server(ctx0, max_batch=64, pool_ciphertexts=1024)
    try:
        ct = keys0.encrypt(np.array([0, 1], dtype=np.uint8))
        with pytest.raises(F.FheaccError):
            srv.submit(ct, [F.AND], [0], [0], 1)      # same node twice
        with pytest.raises(F.FheaccError):
            srv.submit(ct, [F.AND], [0], [2], 1)      # not an earlier node
        with pytest.raises(F.FheaccError):
            srv.submit(ct, [9], [0], [1], 1)          # bad gate code
    finally:
        srv.close()


def test_server_pool_sized_from_free_memory(F, ctx0, keys0):
    """pool_ciphertexts = 0: the pool is sized at creation from the device
    memory then free (a quarter, at most 32 GiB), and serves requests."""
    import torch
    free_b, _ = torch.cuda.mem_get_info()
    srv = F.Server(ctx0, max_batch=256, pool_ciphertexts=0)
    try:
        st = srv.stats()
        ct_bytes = (keys0.P.n + 1) * 8
        assert st["pool_slots"] > 0 and st["lanes"] == 2
        assert st["pool_slots"] * ct_bytes <= min(free_b // 4, 32 << 30)
        assert st["free_slots"] == st["pool_slots"]
        ct, want = make_query(F, keys0, 2, match_at=0, seed=301)
        rid, _ = srv.submit(ct, *F.psi_equality_circuit(2))
        got = wait_all(srv, [rid])
        assert got[rid][0] == F.OK
        assert np.array_equal(keys0.decrypt(got[rid][1]), want)
    finally:
        srv.close()


def test_server_wide_parameter_set(F, ctx1, keys1):
    """The N = 2048, 64-bit set through the server: a small circuit (three
    gates in two levels), each request's words equal to the batched call on the
    same gate inputs, mixed with other requests on both lanes."""
    rng = np.random.default_rng(77)
    reqs = []
    for k in range(4):
        bits = rng.integers(0, 2, 3).astype(np.uint8)
        ct = keys1.encrypt(bits, seed=500 + k)
        # node 3 = NAND(0, 1), node 4 = XOR(3, 2)
        reqs.append((ct, bits))
    srv = F.Server(ctx1, max_batch=64, pool_ciphertexts=256)
    try:
        ids = [srv.submit(ct, [F.NAND, F.XOR], [0, 3], [1, 2], 1)[0] for ct, _ in reqs]
        got = wait_all(srv, ids, timeout_s=300)
        for rid, (ct, bits) in zip(ids, reqs):
            assert got[rid][0] == F.OK
            want = (1 - (bits[0] & bits[1])) ^ bits[2]
            assert keys1.decrypt(got[rid][1])[0] == want
            first = ctx1.eval_bootstrap_batch(ct[0:1], ct[1:2], [F.NAND])
            direct = ctx1.eval_bootstrap_batch(first, ct[2:3], [F.XOR])
            assert np.array_equal(got[rid][1], direct)
    finally:
        srv.close()


@pytest.mark.parametrize("wide", [False, True], ids=["n1024", "n2048"])
def test_server_tiled_keyswitch_rounds(F, cuda_ok, request, wide):
    """A request of one level of independent NAND gates, large enough that its
    round takes the tiled LWE key switch (1024 gates and more at N = 1024, two
    gates per SM at N = 2048), whose outputs go to the server's pool slots
    through an index array: every output word equals the batched call's on the
    same inputs (integer words, bit-exact) and decrypts to the NAND."""
    torch = cuda_ok
    ctx = request.getfixturevalue("ctx1" if wide else "ctx0")
    ks = request.getfixturevalue("keys1" if wide else "keys0")
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    count = 2 * sms + 16 if wide else 1100
    rng = np.random.default_rng(91 + int(wide))
    bits = rng.integers(0, 2, 2 * count).astype(np.uint8)
    ct = ks.encrypt(bits, seed=700 + int(wide))
    gates = [F.NAND] * count
    in1 = list(range(0, 2 * count, 2))
    in2 = list(range(1, 2 * count, 2))
    srv = F.Server(ctx, max_batch=count, pool_ciphertexts=4 * count)
    try:
        rid, _ = srv.submit(ct, gates, in1, in2, count)
        got = wait_all(srv, [rid], timeout_s=300)[rid]
    finally:
        srv.close()
    assert got[0] == F.OK
    direct = ctx.eval_bootstrap_batch(ct[0::2].copy(), ct[1::2].copy(), np.array(gates, dtype=np.int32))
    assert np.array_equal(got[1], direct)
    want = 1 - (bits[0::2] & bits[1::2])
    assert np.array_equal(ks.decrypt(got[1]), want)
