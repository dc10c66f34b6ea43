"""bench.py's multi-GPU path on the CPU: two gloo ranks, each bootstrapping its
own shard of independent gates (no data-path collective), timed with the
barrier and max-over-ranks that the GPU run uses. The shard's gates run
through the oracle here, since the ranks have no GPU."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    import time
    import bench
    from oracle_lib import Oracle, pkg
    F = pkg()
    D = bench.Dist(use_cuda=False)
    P = F.params_preset(0)
    P.n = 16
    F.derive(P)
    lsk, rsk, x, y, c1, c2, gates = bench.make_inputs(F, P, 3, D.rank)
    bt = F.bootstrap_key(P, 13, lsk, rsk)
    ks = F.keyswitch_key(P, 14, rsk, lsk)
    ora = Oracle.from_params(P)
    D.barrier()
    t0 = time.perf_counter()
    out, failed = ora.eval_bootstrap_batch(c1, c2, gates, bt, ks, threads=1)
    dt = time.perf_counter() - t0
    D.barrier()
    slowest = D.max(dt)
    ok = failed == 0 and np.array_equal(F.LWE_decrypt(P, lsk, out), [F.gate_truth(F.NAND, a, b) for a, b in zip(x, y)])
    q.put((D.rank, bool(ok), dt, slowest, int(c1[:, :4].sum() % 1000003)))
    D.close()


def test_two_ranks_shard_and_take_the_slowest(F):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] for r in res)                       # each shard bootstraps correctly
    assert res[0][3] == res[1][3] == max(r[2] for r in res)   # both ranks see the max time
    assert res[0][4] != res[1][4]                       # the shards hold different gates


def test_reference_arm_other_ranks_exit_without_work(F):
    import subprocess
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env, cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""
