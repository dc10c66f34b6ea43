"""The oracle on its own (CPU): its key generation (oracle/fhe_keygen.c, used
by the CPU reference arm of bench.py so that arm loads nothing of the
product) gives keys with which every gate decrypts correctly, and its
issue orders relate as the reference's do: fpga_eval_bootstrap_x1's order
(myfpga.cpp:1037-1046) applies one step more than the CPU path
(RLWE.cpp:754-767) exactly when the first step's residue is 0, and
otherwise gives the CPU path's words."""
import numpy as np
import pytest

from oracle_lib import Oracle


@pytest.fixture(scope="module")
def small():
    o = Oracle.preset(0, n=24)
    lsk, rsk, bt, ks = o.keygen(77, threads=4)
    return o, lsk, bt, ks


def _inputs(o, lsk, count, seed):
    rng = np.random.default_rng(seed)
    x = rng.integers(0, 2, count).astype(np.uint8)
    y = rng.integers(0, 2, count).astype(np.uint8)
    g = rng.integers(0, 6, count).astype(np.int32)
    c = o.lwe_encrypt(seed, lsk, np.concatenate([x, y]))
    return x, y, g, c[:count].copy(), c[count:].copy()


def _truth(g, a, b):
    return [a | b, a & b, 1 - (a | b), 1 - (a & b), a ^ b, 1 - (a ^ b)][g]


def test_oracle_keygen_decrypts_all_gates(small):
    o, lsk, bt, ks = small
    x, y, g, c1, c2 = _inputs(o, lsk, 12, seed=5)
    assert [o.lwe_decrypt(lsk, c) for c in c1] == list(x)
    out, failed = o.eval_bootstrap_batch(c1, c2, g, bt, ks, threads=4)
    assert failed == 0
    assert [o.lwe_decrypt(lsk, c) for c in out] == [_truth(int(a), int(b), int(d)) for a, b, d in zip(g, x, y)]


def test_oracle_x1_order(small):
    o, lsk, bt, ks = small
    x, y, g, c1, c2 = _inputs(o, lsk, 200, seed=6)
    q, Br = int(o.p.q), int(o.p.Br)
    a1, a2 = c1[:, 0].astype(np.int64), c2[:, 0].astype(np.int64)
    a0 = np.where((g == 4) | (g == 5), 2 * (a1 - a2), a1 + a2) % q
    zero = ((q - a0) % q) % Br == 0
    pick = np.concatenate([np.flatnonzero(zero)[:3], np.flatnonzero(~zero)[:3]])
    assert zero[pick].sum() >= 1
    for i in pick:
        acc_cpu, s_cpu = o.blind_rotate(c1[i], c2[i], int(g[i]), bt, fpga_compat=0)
        acc_x1, s_x1 = o.blind_rotate(c1[i], c2[i], int(g[i]), bt, fpga_compat=2)
        assert s_x1 == s_cpu + (1 if zero[i] else 0)
        assert np.array_equal(acc_x1, acc_cpu) != bool(zero[i])
        out, rc = o.eval_bootstrap(c1[i], c2[i], int(g[i]), bt, ks, fpga_compat=2)
        assert rc == 0
        assert o.lwe_decrypt(lsk, out) == _truth(int(g[i]), int(x[i]), int(y[i]))
