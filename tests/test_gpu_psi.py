"""The PSI application's RLWE-level operations on the GPU: CMUX, the RLWE
blind rotation and homo_expand against the oracle (bit-exact), and the
reference's PSI flow (test.cpp:1510-1606: homo_expand, a CMUX tree selecting
a database entry, a blind rotation) end to end with real encryptions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def host(t):
    return t.cpu().numpy().view(np.uint64)


@pytest.mark.parametrize("wide", [False, True])
def test_cmux_vs_oracle(F, request, cuda_ok, wide):
    torch = cuda_ok
    ks = request.getfixturevalue("keys1" if wide else "keys0")
    ctx = request.getfixturevalue("ctx1" if wide else "ctx0")
    P, o = ks.P, ks.oracle
    rw, gw = 2 * P.N, P.digitG * 4 * P.N
    rng = np.random.default_rng(31)
    n = 5
    v = rng.integers(0, P.Q, (2 * n, rw), dtype=np.uint64)
    sel = rng.integers(0, P.Q, (n, gw), dtype=np.uint64)
    dv, ds, out = dev(torch, v), dev(torch, sel), torch.zeros(n * rw, dtype=torch.int64, device="cuda")
    # pairs (v[2k], v[2k+1]) of one array, one RGSW per pair
    ctx.CMUX(dv.data_ptr(), dv.data_ptr() + 8 * rw, ds.data_ptr(), out.data_ptr(), n, in_stride=2 * rw,
             sel_shared=False)
    torch.cuda.synchronize()
    got = host(out).reshape(n, rw)
    for k in range(n):
        assert np.array_equal(got[k], o.cmux(v[2 * k], v[2 * k + 1], sel[k]))
    # contiguous c0 / c1, shared RGSW, output over c0
    c0, c1 = dev(torch, v[:n]), dev(torch, v[n:])
    ctx.CMUX(c0.data_ptr(), c1.data_ptr(), ds.data_ptr(), c0.data_ptr(), n)
    torch.cuda.synchronize()
    got = host(c0).reshape(n, rw)
    for k in range(n):
        assert np.array_equal(got[k], o.cmux(v[k], v[n + k], sel[0]))


@pytest.mark.parametrize("wide", [False, True])
def test_rlwe_blind_rotate_vs_oracle(F, request, cuda_ok, wide):
    torch = cuda_ok
    ks = request.getfixturevalue("keys1" if wide else "keys0")
    ctx = request.getfixturevalue("ctx1" if wide else "ctx0")
    P, o = ks.P, ks.oracle
    rw, gw, logN = 2 * P.N, P.digitG * 4 * P.N, P.N.bit_length() - 1
    rng = np.random.default_rng(32)
    c = rng.integers(0, P.Q, (2, rw), dtype=np.uint64)
    rg = rng.integers(0, P.Q, logN * gw, dtype=np.uint64)
    dc, dr = dev(torch, c), dev(torch, rg)
    for fwd in (False, True):
        out = torch.zeros(2 * rw, dtype=torch.int64, device="cuda")
        ctx.blind_rotate_RLWE(dc.data_ptr(), dr.data_ptr(), fwd, out.data_ptr(), 2)
        torch.cuda.synchronize()
        got = host(out).reshape(2, rw)
        for k in range(2):
            assert np.array_equal(got[k], o.rlwe_blind_rotate(c[k], fwd, rg))


def test_homo_expand_vs_oracle(F, ctx0, keys0, cuda_ok):
    torch = cuda_ok
    P, o = keys0.P, keys0.oracle
    ctx0.upload_subs_key(keys0.subs)
    rw, gw = 2 * P.N, P.digitG * 4 * P.N
    rng = np.random.default_rng(33)
    packed = rng.integers(0, P.Q, P.digitG * rw, dtype=np.uint64)
    enc = rng.integers(0, P.Q, gw, dtype=np.uint64)
    out = torch.zeros(P.N * gw, dtype=torch.int64, device="cuda")
    dp, de = dev(torch, packed), dev(torch, enc)   # kept alive while the device reads them
    ctx0.homo_expand(dp.data_ptr(), de.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(host(out).reshape(P.N, gw), o.homo_expand(packed, enc, keys0.subs))


def test_psi_flow_end_to_end(F, ctx1, keys1, cuda_ok):
    """test.cpp:1510-1606 at N = 2048: the packed query sets every odd bit, so
    the tree (levels 11..17) selects database entry 0b1010101 = 85 and the
    blind rotation (RGSWs 0..10) rotates by X^-682; the entry holds Q/2 in
    coefficients 0..85, so the result decrypts to ones at 1366..1451."""
    torch = cuda_ok
    P, o, sk = keys1.P, keys1.oracle, keys1.rlwe_sk
    N, Q, dG = P.N, P.Q, P.digitG
    rw, gw, logN = 2 * N, dG * 4 * N, 11
    ctx1.upload_subs_key(keys1.subs)
    s_time = o.intt(sk)
    enc_neg_s = F.RGSW_encrypt(P, 41, sk, o.ntt((Q - s_time) % Q))
    packed, pow_bg = [], 1
    iN = pow(N, Q - 2, Q)
    for i in range(dG):
        m = np.zeros(N, dtype=np.uint64)
        m[1::2] = pow_bg * iN % Q
        packed.append(F.RLWE_encrypt(P, 100 + i, sk, o.ntt(m)))
        pow_bg = pow_bg * (1 << P.BG_bits) % Q
    rgsw = torch.zeros(N * gw, dtype=torch.int64, device="cuda")
    dp, de = dev(torch, np.concatenate(packed)), dev(torch, enc_neg_s)
    ctx1.homo_expand(dp.data_ptr(), de.data_ptr(), rgsw.data_ptr())
    entries = 1 << (18 - logN)
    db = []
    for i in range(entries):
        m = np.zeros(N, dtype=np.uint64)
        m[:i + 1] = Q // 2
        db.append(F.RLWE_encrypt(P, 1000 + i, sk, o.ntt(m)))
    bufs = [dev(torch, np.concatenate(db)), torch.zeros(entries // 2 * rw, dtype=torch.int64, device="cuda"),
            torch.zeros(entries // 2 * rw, dtype=torch.int64, device="cuda")]
    src, count, level = bufs[0], entries, logN
    while count > 1:   # v[k] = CMUX(v[2k], v[2k+1], RGSW[level])
        dst = bufs[1 + (level & 1)]
        ctx1.CMUX(src.data_ptr(), src.data_ptr() + 8 * rw, rgsw.data_ptr() + 8 * gw * level, dst.data_ptr(),
                  count // 2, in_stride=2 * rw)
        src, count, level = dst, count // 2, level + 1
    out = torch.zeros(rw, dtype=torch.int64, device="cuda")
    ctx1.blind_rotate_RLWE(src.data_ptr(), rgsw.data_ptr(), False, out.data_ptr(), 1)
    torch.cuda.synchronize()
    phase = F.RLWE_phase(P, sk, host(out))
    bits = ((2 * phase.astype(object) + Q // 2) // Q % 2).astype(np.uint8)
    want = np.zeros(N, dtype=np.uint8)
    want[1366:1452] = 1
    assert np.array_equal(bits, want)
