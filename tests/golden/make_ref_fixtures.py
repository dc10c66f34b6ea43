"""Runs the reference's own eval_bootstrap (oracle/_ref/libref.so, built from the
reference sources by oracle/build_ref.sh) on keys and ciphertexts generated
from fixed seeds by this package, and stores the outputs as a fixture.

The GPU test test_reference_fixture (tests/test_gpu_bootstrap.py) regenerates
the same keys from the same seeds (the generator is integer-only, so every
machine gets the same words) and compares the GPU outputs with these
reference outputs; test_oracle_equals_reference_outputs checks the oracle.

Run here, where the reference is mounted:
    python tests/golden/make_ref_fixtures.py
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


def main():
    if not ref_available():
        sys.exit("oracle/_ref/libref.so not built (oracle/build_ref.sh)")
    F = pkg()
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
                        inputs_sha256=np.bytes_(digest(c1, c2)),
                        keys_sha256=np.bytes_(digest(ks.lwe_sk, ks.rlwe_sk, ks.btkey[:1 << 20], ks.kskey[:1 << 20])),
                        seeds=np.array([SEEDS[k] for k in ("lwe_sk", "rlwe_sk", "btkey", "kskey")]))
    print("wrote ref_bootstrap_p0.npz")


if __name__ == "__main__":
    main()
