"""The automorphism, the RLWE key switch and expand_RLWE on the GPU against
the reference's golden RLWESUBS transcript (N=2048, Q < 2^54) and the oracle
(both word widths), bit-exact."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


def test_rlwesubs_golden_transcript(F, ctx1, keys1, cuda_ok):
    """RLWESUBS_output.txt: RLWE_substitute(f=0) then RLWE_keyswitch."""
    torch = cuda_ok
    g = np.load(os.path.join(GOLD, "rlwesubs_2k.npz"))
    assert int(g["Q"]) == keys1.P.Q and int(g["N"]) == keys1.P.N
    inp, ksk = dev(torch, g["inp"]), dev(torch, g["ksk"].reshape(-1))
    sub = torch.zeros(4096, dtype=torch.int64, device="cuda")
    ctx1.rlwe_substitute_async(inp.data_ptr(), 1, 0, sub.data_ptr())
    out = torch.zeros_like(sub)
    ctx1.rlwe_keyswitch_async(sub.data_ptr(), 1, ksk.data_ptr(), out.data_ptr())
    ctx1.sync()
    assert np.array_equal(host(sub), g["subs"])
    assert np.array_equal(host(out), g["out"])


@pytest.mark.parametrize("wide", [False, True])
def test_substitute_and_keyswitch_vs_oracle(F, request, cuda_ok, wide):
    torch = cuda_ok
    ks = request.getfixturevalue("keys1" if wide else "keys0")
    ctx = request.getfixturevalue("ctx1" if wide else "ctx0")
    o, P = ks.oracle, ks.P
    rng = np.random.default_rng(11)
    c = rng.integers(0, P.Q, (3, 2 * P.N), dtype=np.uint64)
    c[0, :5] = [0, 1, P.Q - 1, 2, 3]
    dc = dev(torch, c)
    logN = P.N.bit_length() - 1
    for f in (0, 3, logN - 1):
        out = torch.zeros_like(dc)
        ctx.rlwe_substitute_async(dc.data_ptr(), 3, f, out.data_ptr())
        ctx.sync()
        assert np.array_equal(host(out), np.stack([o.rlwe_substitute(x, f) for x in c])), f
    ksk = rng.integers(0, P.Q, (int(P.digitKS_R), 2, P.N), dtype=np.uint64)
    dk = dev(torch, ksk.reshape(-1))
    out = torch.zeros_like(dc)
    ctx.rlwe_keyswitch_async(dc.data_ptr(), 3, dk.data_ptr(), out.data_ptr())
    ctx.sync()
    assert np.array_equal(host(out), np.stack([o.rlwe_keyswitch(x, ksk) for x in c]))


@pytest.mark.parametrize("wide", [False, True])
def test_subs_keyswitch_and_expand_vs_oracle(F, request, cuda_ok, wide):
    torch = cuda_ok
    ks = request.getfixturevalue("keys1" if wide else "keys0")
    ctx = request.getfixturevalue("ctx1" if wide else "ctx0")
    o, P = ks.oracle, ks.P
    ctx.upload_subs_key(ks.subs)
    rng = np.random.default_rng(12)
    c = rng.integers(0, P.Q, (2, 2 * P.N), dtype=np.uint64)
    dc = dev(torch, c)
    kw = int(P.digitKS_R) * 2 * P.N
    for f in (0, 5):
        out = torch.zeros_like(dc)
        ctx.subs_keyswitch_async(dc.data_ptr(), 2, f, out.data_ptr())
        ctx.sync()
        want = np.stack([o.rlwe_keyswitch(o.rlwe_substitute(x, f), ks.subs[f * kw:(f + 1) * kw]) for x in c])
        assert np.array_equal(host(out), want)
    # expand_RLWE of an encryption of a polynomial with small coefficients
    msg = np.zeros(P.N, dtype=np.uint64)
    msg[:8] = [1, 0, 1, 1, 0, 0, 1, 0]
    m_ntt = o.ntt(msg * np.uint64(P.Q // 8))
    ct = F.RLWE_encrypt(P, 77, ks.rlwe_sk, m_ntt)
    exp = torch.zeros((P.N, 2 * P.N), dtype=torch.int64, device="cuda")
    dct = dev(torch, ct)
    ctx.expand_RLWE(dct.data_ptr(), exp.data_ptr())
    ctx.sync()
    assert np.array_equal(host(exp), o.expand_rlwe(ct, ks.subs))
