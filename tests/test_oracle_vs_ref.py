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
