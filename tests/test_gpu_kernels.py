"""GPU sub-steps against the oracle and the reference's golden transcripts:
NTT / inverse NTT, RLWE x RGSW, blind rotation, LWE key switch, modulus
switch. All comparisons are bit-exact."""
import os

import numpy as np
import pytest

from conftest import random_gate_batch
from oracle_lib import Oracle

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


@pytest.fixture(scope="module")
def ctx_golden(F, cuda_ok):
    P = F.params_preset(2)   # N=1024, Q=0x7FFF801, BG=2^9 x3: the transcript's set
    ctx = F.Context(P, 0)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("count", [1, 7, 64])
def test_ntt_forward_inverse(F, ctx0, keys0, cuda_ok, count):
    torch = cuda_ok
    o = keys0.oracle
    rng = np.random.default_rng(count)
    Q = keys0.P.Q
    a = rng.integers(0, Q, (count, 1024), dtype=np.uint64)
    a[0, :8] = [0, 1, Q - 1, Q - 2, 2, 3, Q // 2, Q // 2 + 1]   # edge values
    d = dev(torch, a)
    ctx0.ntt_forward(d.data_ptr(), count)
    torch.cuda.synchronize()
    got = host(d)
    want = np.stack([o.ntt(x) for x in a])
    assert np.array_equal(got, want)
    ctx0.ntt_inverse(d.data_ptr(), count)
    torch.cuda.synchronize()
    assert np.array_equal(host(d), a)
    # inverse of arbitrary NTT-domain input
    d2 = dev(torch, a)
    ctx0.ntt_inverse(d2.data_ptr(), count)
    torch.cuda.synchronize()
    assert np.array_equal(host(d2), np.stack([o.intt(x) for x in a]))


def test_rlwe_mult_rgsw_golden(F, ctx_golden, cuda_ok):
    torch = cuda_ok
    g = np.load(os.path.join(GOLD, "rlwe_x_rgsw_1k.npz"))
    acc = dev(torch, g["acc"])
    rgsw = dev(torch, g["rgsw"].reshape(-1))
    out = torch.zeros(2048, dtype=torch.int64, device="cuda")
    ctx_golden.rlwe_mult_rgsw(acc.data_ptr(), rgsw.data_ptr(), out.data_ptr(), 1)
    torch.cuda.synchronize()
    assert np.array_equal(host(out), g["out"])


def test_rlwe_mult_rgsw_random(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    o = keys0.oracle
    rng = np.random.default_rng(5)
    Q = keys0.P.Q
    count = 9
    acc = rng.integers(0, Q, (count, 2048), dtype=np.uint64)
    acc[0] = Q - 1    # largest digits everywhere
    rgsw = rng.integers(0, Q, (count, 4 * 4 * 1024), dtype=np.uint64)
    rgsw[1] = Q - 1
    out = torch.zeros((count, 2048), dtype=torch.int64, device="cuda")
    da, dr = dev(torch, acc), dev(torch, rgsw)   # keep the inputs alive until the kernel has run
    ctx0.rlwe_mult_rgsw(da.data_ptr(), dr.data_ptr(), out.data_ptr(), count)
    torch.cuda.synchronize()
    want = np.stack([o.rlwe_mult_rgsw(acc[i], rgsw[i]) for i in range(count)])
    assert np.array_equal(host(out), want)


def test_blind_rotate_vs_oracle(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    x, y, g, c1, c2 = random_gate_batch(keys0, 6, seed=21, gates=[0, 1, 2, 3, 4, 5])
    acc = torch.zeros((6, 2048), dtype=torch.int64, device="cuda")
    dg = torch.from_numpy(g).cuda()
    d1, d2 = dev(torch, c1), dev(torch, c2)
    ctx0.blind_rotate_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 6, acc.data_ptr())
    ctx0.sync()
    got = host(acc)
    for i in range(6):
        want, steps = keys0.oracle.blind_rotate(c1[i], c2[i], int(g[i]), keys0.btkey)
        assert steps > 900
        assert np.array_equal(got[i], want), "gate %d" % i


def test_lwe_keyswitch_and_modswitch(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    o = keys0.oracle
    rng = np.random.default_rng(9)
    Q = keys0.P.Q
    count = 5
    rlwe = rng.integers(0, Q, (count, 2048), dtype=np.uint64)
    out = torch.zeros((count, keys0.P.n + 1), dtype=torch.int64, device="cuda")
    dr = dev(torch, rlwe)
    ctx0.lwe_keyswitch_async(dr.data_ptr(), count, out.data_ptr())
    ctx0.sync()
    ks = host(out)
    want = np.stack([o.lwe_keyswitch(rlwe[i], keys0.kskey) for i in range(count)])
    assert np.array_equal(ks, want)
    ms = torch.zeros_like(out)
    ctx0.lwe_modswitch_async(out.data_ptr(), count, ms.data_ptr())
    ctx0.sync()
    assert np.array_equal(host(ms), np.stack([o.lwe_modswitch(w) for w in want]))
    # edge words of the modulus switch: 0, Q-1 (rounds to q, not reduced)
    edge = np.zeros((1, keys0.P.n + 1), dtype=np.uint64)
    edge[0, :4] = [0, Q - 1, Q // 2, 1]
    de = dev(torch, edge)
    me = torch.zeros_like(de)
    ctx0.lwe_modswitch_async(de.data_ptr(), 1, me.data_ptr())
    ctx0.sync()
    assert np.array_equal(host(me)[0], o.lwe_modswitch(edge[0]))
    assert host(me)[0, 1] == keys0.P.q


@pytest.mark.gpu
def test_throughput_probes(F, ctx0, cuda_ok):
    """The roofline probes run on the device and give plausible figures: an
    IMAD rate within a factor of a few of 64 lanes per SM per clock, and NTT /
    MAC SM times in the hundreds of ns."""
    imad = ctx0.measure_imad_rate()
    assert 1e12 < imad < 1e14
    comp = ctx0.measure_components()
    for k in ("ntt_fwd", "ntt_digit", "intt", "mac"):
        assert 10.0 < comp[k] < 100000.0, comp
    # the table-driven first stages make the digit transform no slower
    assert comp["ntt_digit"] < 1.2 * comp["ntt_fwd"], comp
