"""Pins the oracle against the reference's own runtime compiled here
(oracle/_ref/libref.so from oracle/build_ref.sh). Skipped where the
reference is not mounted (the library is not built there)."""
import numpy as np
import pytest

from oracle_lib import Oracle, Ref, ref_available

pytestmark = pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (reference not mounted)")


@pytest.fixture(scope="module")
def pair(keys0):
    o = keys0.oracle
    return o, Ref(o)


def test_tables_and_ntt(pair):
    o, r = pair
    for a, b in zip(o.tables(), r.tables()):
        assert np.array_equal(a, b)
    rng = np.random.default_rng(0)
    for _ in range(5):
        a = rng.integers(0, o.p.Q, o.N, dtype=np.uint64)
        assert np.array_equal(o.ntt(a), r.ntt(a))
        assert np.array_equal(o.intt(a), r.intt(a))


def test_rlwe_mult_rgsw(pair):
    o, r = pair
    rng = np.random.default_rng(1)
    for _ in range(3):
        acc = rng.integers(0, o.p.Q, 2 * o.N, dtype=np.uint64)
        rgsw = rng.integers(0, o.p.Q, int(o.p.digitG) * 4 * o.N, dtype=np.uint64)
        assert np.array_equal(o.rlwe_mult_rgsw(acc, rgsw), r.rlwe_mult_rgsw(acc, rgsw))


def test_acc_initialization(pair):
    o, r = pair
    q = o.p.q
    for gate in range(6):
        b1 = o.p.gate_constant[gate] % q
        for value in (0, 1, 100, 255, 256, 511):
            a = o.acc_initialization(2 * o.N // q, b1, (b1 + q // 2) % q, value)
            assert np.array_equal(a, r.acc_initialization(2 * o.N // q, b1, (b1 + q // 2) % q, value))


def test_keyswitch_modswitch(pair, keys0):
    o, r = pair
    r.load_keys(keys0.btkey, keys0.kskey)
    rng = np.random.default_rng(2)
    for _ in range(2):
        rl = rng.integers(0, o.p.Q, 2 * o.N, dtype=np.uint64)
        k1 = o.lwe_keyswitch(rl, keys0.kskey)
        assert np.array_equal(k1, r.lwe_keyswitch(rl))
        assert np.array_equal(o.lwe_modswitch(k1), r.lwe_modswitch(k1))


def test_eval_bootstrap(pair, keys0):
    o, r = pair
    r.load_keys(keys0.btkey, keys0.kskey)
    c = keys0.encrypt(np.array([1, 0, 1, 1], dtype=np.uint8), seed=9)
    for gate, (i, j) in zip((3, 4), ((0, 1), (2, 3))):
        a, rc1 = o.eval_bootstrap(c[i], c[j], gate, keys0.btkey, keys0.kskey)
        b, rc2 = r.eval_bootstrap(c[i], c[j], gate)
        assert rc1 == rc2 == 0
        assert np.array_equal(a, b)
    # c1 == c2: the reference exits; both entry points here report it
    assert o.eval_bootstrap(c[0], c[0], 3, keys0.btkey, keys0.kskey)[1] == -1
    assert r.eval_bootstrap(c[0], c[0], 3)[1] == -1
    r.free_keys()


def test_substitute_keyswitch_expand(F, keys0):
    """RLWE_substitute, RLWE_keyswitch and expand_RLWE at N=1024. (The
    reference builds its rotation polys for N >= 1024 only: rotate_vector_gen,
    params.cpp:177-210, indexes N - 2^j for j < 11.)"""
    P = keys0.P
    o = keys0.oracle
    r = Ref(o)
    subs = keys0.subs
    rng = np.random.default_rng(4)
    c = rng.integers(0, P.Q, 2 * P.N, dtype=np.uint64)
    kw = int(P.digitKS_R) * 2 * P.N
    for f in (0, 3, 9):
        s1 = o.rlwe_substitute(c, f)
        assert np.array_equal(s1, r.rlwe_substitute(c, f))
        assert np.array_equal(o.rlwe_keyswitch(s1, subs[f * kw:(f + 1) * kw]),
                              r.rlwe_keyswitch(s1, subs[f * kw:(f + 1) * kw]))
    assert np.array_equal(o.expand_rlwe(c, subs), r.expand_rlwe(c, subs))


def test_cmux_and_homo_expand(F, keys0, pair):
    """CMUX (RLWE.cpp:788-793) and homo_expand (app.cpp:78-96) at N=1024 on
    uniform words (parity of the arithmetic; decryption is checked on the GPU)."""
    o, r = pair
    P = keys0.P
    rng = np.random.default_rng(6)
    rw, gw = 2 * P.N, int(P.digitG) * 4 * P.N
    c0, c1 = rng.integers(0, P.Q, (2, rw), dtype=np.uint64)
    sel = rng.integers(0, P.Q, gw, dtype=np.uint64)
    assert np.array_equal(o.cmux(c0, c1, sel), r.cmux(c0, c1, sel))
    packed = rng.integers(0, P.Q, int(P.digitG) * rw, dtype=np.uint64)
    enc = rng.integers(0, P.Q, gw, dtype=np.uint64)
    assert np.array_equal(o.homo_expand(packed, enc, keys0.subs), r.homo_expand(packed, enc, keys0.subs))


def _blind_rotate_2k(q):
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path[:0] = [here, os.path.dirname(here)]
    from oracle_lib import Oracle, Ref, pkg
    F = pkg()
    P = F.params_preset(1)
    o = Oracle.from_params(P)
    r = Ref(o)
    rng = np.random.default_rng(8)
    c = rng.integers(0, P.Q, 2 * P.N, dtype=np.uint64)
    rg = rng.integers(0, P.Q, 11 * int(P.digitG) * 4 * P.N, dtype=np.uint64)
    ok = []
    for fwd in (False, True):
        ref, rc = r.blind_rotate(c, fwd, rg, 11)
        ok.append(rc == 0 and np.array_equal(o.rlwe_blind_rotate(c, fwd, rg), ref))
    q.put(ok)


def test_rlwe_blind_rotate_2k(F):
    """blind_rotate (RLWE.cpp:824-838) at N=2048, the size its fixed count of
    11 rotations (params.h num_rotate_poly) is written for; in a separate
    process, as the reference keeps one parameter set in its globals."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    pr = ctx.Process(target=_blind_rotate_2k, args=(q,))
    pr.start()
    ok = q.get(timeout=600)
    pr.join(timeout=60)
    assert pr.exitcode == 0 and ok == [True, True]
