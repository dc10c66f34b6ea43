"""Runs the reference's own eval_bootstrap (oracle/_ref/libref.so, built from the
reference sources by oracle/build_ref.sh) on keys and ciphertexts generated
from fixed seeds by this package, and stores the outputs as a fixture.

The GPU test test_reference_fixture (tests/test_gpu_bootstrap.py) regenerates
the same keys from the same seeds (the generator is integer-only, so every
machine gets the same words) and compares the GPU outputs with these
reference outputs; test_oracle_equals_reference_outputs checks the oracle.

Fixtures: ref_bootstrap_p0.npz (N = 1024, 27-bit Q) and ref_bootstrap_p1.npz
(N = 2048, 54-bit Q: bootstraps, LWE_keyswitch and LWE_modswitch). Run here,
where the reference is mounted:
    python tests/golden/make_ref_fixtures.py [p0] [p1]
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
sys.path.insert(0, TESTS)

from conftest import SEEDS, KeySet  # noqa: E402
from oracle_lib import Ref, pkg, ref_available  # noqa: E402


def truth_table_inputs(ks):
    xs, ys, gs = [], [], []
    for g in range(6):
        for a in (0, 1):
            for b in (0, 1):
                xs.append(a); ys.append(b); gs.append(g)
    x = np.array(xs, dtype=np.uint8); y = np.array(ys, dtype=np.uint8); g = np.array(gs, dtype=np.int32)
    c = ks.encrypt(np.concatenate([x, y]), seed=77)
    return x, y, g, c[:24].copy(), c[24:].copy()


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def keys_digest(ks):
    return digest(ks.lwe_sk, ks.rlwe_sk, ks.btkey[:1 << 20], ks.kskey[:1 << 20])


def fixture_p0(F):
    ks = KeySet(F, 0)
    x, y, g, c1, c2 = truth_table_inputs(ks)
    ref = Ref(ks.oracle)
    ref.load_keys(ks.btkey, ks.kskey)
    out = np.zeros((24, ks.P.n + 1), dtype=np.uint64)
    for i in range(24):
        o, rc = ref.eval_bootstrap(c1[i], c2[i], int(g[i]))
        assert rc == 0
        out[i] = o
    ref.free_keys()
    assert out.max() <= ks.P.q
    np.savez_compressed(os.path.join(HERE, "ref_bootstrap_p0.npz"), x=x, y=y, gates=g, out=out.astype(np.uint16),
                        inputs_sha256=np.bytes_(digest(c1, c2)), keys_sha256=np.bytes_(keys_digest(ks)),
                        seeds=np.array([SEEDS[k] for k in ("lwe_sk", "rlwe_sk", "btkey", "kskey")]))
    print("wrote ref_bootstrap_p0.npz")


# The 64-bit set (N = 2048, Q = 18014398509404161 < 2^54, BG = 2^9 x 6,
# Bks = 25 x 12): the truth tables at a reduced LWE dimension, the reference's
# LWE_keyswitch and LWE_modswitch on stored random inputs (edge words included),
# and four gates at the full n = 630.
P1_SMALL_N = 32
P1_FULL_GATES = [(3, 1, 1), (1, 1, 0), (4, 0, 1), (5, 1, 1)]   # (gate, x, y): NAND, AND, XOR, XNOR


def keyswitch_inputs(P, seed=2054):
    """Two random NTT-domain RLWEs and one with edge words (0, 1, Q-1, Q/2)."""
    Q = int(P.Q)
    rng = np.random.default_rng(seed)
    rl = rng.integers(0, Q, (3, 2 * P.N), dtype=np.uint64)
    rl[2, :8] = [0, 1, Q - 1, Q // 2, Q // 2 + 1, 0, Q - 1, 2]
    rl[2, P.N:P.N + 4] = [0, Q - 1, Q // 2, 1]
    lw = rng.integers(0, Q, (4, P.n + 1), dtype=np.uint64)
    lw[3, :6] = [0, 1, Q - 1, Q // 2, Q // 2 + 1, Q // 1024]
    return rl, lw


def full_inputs(ks):
    x = np.array([a for _, a, _ in P1_FULL_GATES], dtype=np.uint8)
    y = np.array([b for _, _, b in P1_FULL_GATES], dtype=np.uint8)
    g = np.array([t for t, _, _ in P1_FULL_GATES], dtype=np.int32)
    c = ks.encrypt(np.concatenate([x, y]), seed=78)
    k = len(x)
    return x, y, g, c[:k].copy(), c[k:].copy()


def fixture_p1(F):
    small = KeySet(F, 1, n=P1_SMALL_N)
    x, y, g, c1, c2 = truth_table_inputs(small)
    ref = Ref(small.oracle)
    ref.load_keys(small.btkey, small.kskey)
    out = np.zeros((24, small.P.n + 1), dtype=np.uint64)
    for i in range(24):
        o, rc = ref.eval_bootstrap(c1[i], c2[i], int(g[i]))
        assert rc == 0
        out[i] = o
    rl, lw = keyswitch_inputs(small.P)
    ks_out = np.stack([ref.lwe_keyswitch(r) for r in rl])
    ms_out = np.stack([ref.lwe_modswitch(v) for v in lw])
    ref.free_keys()
    # the restatement agrees before anything is stored
    o_out, failed = small.oracle.eval_bootstrap_batch(c1, c2, g, small.btkey, small.kskey)
    assert failed == 0 and np.array_equal(o_out, out)
    assert np.array_equal(np.stack([small.oracle.lwe_keyswitch(r, small.kskey) for r in rl]), ks_out)
    assert np.array_equal(np.stack([small.oracle.lwe_modswitch(v) for v in lw]), ms_out)

    full = KeySet(F, 1)
    fx, fy, fg, f1, f2 = full_inputs(full)
    ref = Ref(full.oracle)
    ref.load_keys(full.btkey, full.kskey)
    fout = np.zeros((len(fx), full.P.n + 1), dtype=np.uint64)
    for i in range(len(fx)):
        o, rc = ref.eval_bootstrap(f1[i], f2[i], int(fg[i]))
        assert rc == 0
        fout[i] = o
    ref.free_keys()
    assert out.max() <= small.P.q and fout.max() <= full.P.q
    np.savez_compressed(os.path.join(HERE, "ref_bootstrap_p1.npz"),
                        x=x, y=y, gates=g, out=out.astype(np.uint16), n_small=np.int32(P1_SMALL_N),
                        inputs_sha256=np.bytes_(digest(c1, c2)), keys_sha256=np.bytes_(keys_digest(small)),
                        ks_in=rl, ks_out=ks_out, ms_in=lw, ms_out=ms_out,
                        full_x=fx, full_y=fy, full_gates=fg, full_out=fout.astype(np.uint16),
                        full_inputs_sha256=np.bytes_(digest(f1, f2)), full_keys_sha256=np.bytes_(keys_digest(full)),
                        seeds=np.array([SEEDS[k] for k in ("lwe_sk", "rlwe_sk", "btkey", "kskey")]))
    print("wrote ref_bootstrap_p1.npz")


def main():
    if not ref_available():
        sys.exit("oracle/_ref/libref.so not built (oracle/build_ref.sh)")
    F = pkg()
    which = sys.argv[1:] or ["p0", "p1"]
    if "p0" in which:
        fixture_p0(F)
    if "p1" in which:
        fixture_p1(F)


if __name__ == "__main__":
    main()
