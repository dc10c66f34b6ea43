"""Pins the oracle (oracle/fhe_oracle.c) against the reference's own golden
data: the RLWE x RGSW and RLWE-substitute transcripts and the parameter files
of cl_fhe_acc/verif/tests/mem_init_content (fixtures made by
tests/golden/make_golden.py)."""
import json
import os

import numpy as np
import pytest

from oracle_lib import Oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def g1k():
    return np.load(os.path.join(GOLD, "rlwe_x_rgsw_1k.npz"))


@pytest.fixture(scope="module")
def g2k():
    return np.load(os.path.join(GOLD, "rlwesubs_2k.npz"))


@pytest.fixture(scope="module")
def o1k(g1k):
    # the transcript's set: N=1024, Q=0x7FFF801, BG=2^9, digitG=3
    return Oracle(n=512, q=512, N=1024, Q=int(g1k["Q"]), BGbits=9, digitG=3, Br=23, digitR=2, Bks=25, digitKS=6,
                  Bks_R_bits=9, digitKS_R=3)


@pytest.fixture(scope="module")
def o2k(g2k):
    return Oracle(n=630, q=512, N=2048, Q=int(g2k["Q"]), BGbits=9, digitG=6, Br=23, digitR=2, Bks=25,
                  digitKS=12, Bks_R_bits=9, digitKS_R=6)


def test_params_files(o1k, o2k):
    with open(os.path.join(GOLD, "params.json")) as f:
        ref = json.load(f)
    for o, tag in ((o1k, "1k"), (o2k, "2k")):
        assert o.p.Q == ref[tag]["Q"]
        assert o.p.iN == ref[tag]["iN"]
        assert o.p.ROU == ref[tag]["ROU"]


def test_find_Q(o1k):
    # Q = previous_prime(first_prime(nbit, N), N), fhe_wo_fpga.cpp:89
    assert o1k.L.ora_find_Q(27, 1024) == 134215681
    assert o1k.L.ora_find_Q(54, 2048) == 18014398509404161


def test_rlwe_mult_rgsw_golden(o1k, g1k):
    assert np.array_equal(o1k.rlwe_mult_rgsw(g1k["acc"], g1k["rgsw"]), g1k["out"])


def test_intt_golden(o1k, g1k):
    acc = g1k["acc"]
    t = np.concatenate([o1k.intt(acc[:1024]), o1k.intt(acc[1024:])])
    assert np.array_equal(t, g1k["acc_time"])
    # round trip back
    f = np.concatenate([o1k.ntt(t[:1024]), o1k.ntt(t[1024:])])
    assert np.array_equal(f, acc)


def test_digit_decompose_golden(o1k, g1k):
    assert np.array_equal(o1k.digit_decompose(g1k["acc"], 3, 9), g1k["dec"])


def test_acc_initialization_golden(o1k, g1k):
    # README.txt beside the transcript: init value 0, bound1 = 3/8*512,
    # bound2 = (bound1 + 512) % 512 ... with embed 2N/q = 4
    b1 = 3 * 512 // 8
    assert np.array_equal(o1k.acc_initialization(4, b1, (b1 + 256) % 512, 0), g1k["acc"])
    t = g1k["acc_time"]
    assert set(np.unique(t[1024:]).tolist()) <= {0, int(g1k["Q8"]), int(g1k["negQ8"])}


def test_substitute_golden(o2k, g2k):
    assert np.array_equal(o2k.rlwe_substitute(g2k["inp"], 0), g2k["subs"])
    t = np.concatenate([o2k.intt(g2k["inp"][:2048]), o2k.intt(g2k["inp"][2048:])])
    assert np.array_equal(t, g2k["inp_time"])


def test_rlwe_keyswitch_golden(o2k, g2k):
    assert np.array_equal(o2k.rlwe_keyswitch(g2k["subs"], g2k["ksk"]), g2k["out"])
    d = o2k.digit_decompose(g2k["subs"], 6, 9)
    assert np.array_equal(d[:, 0, :], g2k["dec"])


def test_ntt_known_answers(o1k):
    """verify_NTT-style checks (test.cpp:137-278): round trip and the
    negacyclic convolution property X^(N-1) * X = -1."""
    rng = np.random.default_rng(1)
    Q, N = o1k.p.Q, o1k.N
    a = rng.integers(0, Q, N, dtype=np.uint64)
    assert np.array_equal(o1k.intt(o1k.ntt(a)), a)
    x1 = np.zeros(N, dtype=np.uint64); x1[1] = 1
    xn = np.zeros(N, dtype=np.uint64); xn[N - 1] = 1
    prod = (o1k.ntt(x1).astype(object) * o1k.ntt(xn).astype(object)) % Q
    res = o1k.intt(np.array(prod, dtype=np.uint64))
    want = np.zeros(N, dtype=np.uint64); want[0] = Q - 1
    assert np.array_equal(res, want)
